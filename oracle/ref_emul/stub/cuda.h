/* Emulation stand-in for <cuda.h> -- test infrastructure only. */
#include "../emu_cuda.h"
