/* Host stand-in for <device_launch_parameters.h> (see cuda_runtime.h in this folder). */
#include "cuda_runtime.h"
