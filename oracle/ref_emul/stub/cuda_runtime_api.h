/* Emulation stand-in for <cuda_runtime_api.h> -- test infrastructure only. */
#include "../emu_cuda.h"
