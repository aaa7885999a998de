// Batched lattice step kernels of the BF16 population storage (see batch_step.cuh).
#include "fsi_gb300.h"
#define FSI_BATCH_STEP_STORAGE FSI_STORAGE_BF16
#define FSI_BATCH_STEP_NAME batch_step_launch_bf16
#include "batch_step.cuh"
