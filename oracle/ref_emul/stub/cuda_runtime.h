/* Emulation stand-in for <cuda_runtime.h> -- test infrastructure only. */
#include "../emu_cuda.h"
