/* Forwarding header so callers that include "fftfpga/fftfpga.h", the
 * reference's include path (api/include/fftfpga/fftfpga.h), build unchanged. */
#include "../fftfpga.h"
