/* Emulation stand-in for <cublas_v2.h> -- test infrastructure only. */
#include "../emu_cuda.h"
