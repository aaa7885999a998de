// Batched lattice step kernels of the F16 population storage (see batch_step.cuh).
#include "fsi_gb300.h"
#define FSI_BATCH_STEP_STORAGE FSI_STORAGE_F16
#define FSI_BATCH_STEP_NAME batch_step_launch_f16
#include "batch_step.cuh"
