// Batched lattice step kernels of the F32 population storage (see batch_step.cuh).
#include "fsi_gb300.h"
#define FSI_BATCH_STEP_STORAGE FSI_STORAGE_F32
#define FSI_BATCH_STEP_NAME batch_step_launch_f32
#include "batch_step.cuh"
