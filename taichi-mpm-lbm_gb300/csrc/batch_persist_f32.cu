// Persistent coupled-step kernel of a batch with F32 population storage (see batch_persistent.cuh).
#define FSI_LAUNCH_RO
#include "fsi_gb300.h"
#define FSI_BATCH_STEP_STORAGE FSI_STORAGE_F32
#define FSI_BATCH_PERSIST_NAME batch_persist_launch_f32
#include "batch_persistent.cuh"
