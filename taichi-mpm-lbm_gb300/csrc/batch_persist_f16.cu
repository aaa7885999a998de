// Persistent coupled-step kernel of a batch with F16 population storage (see batch_persistent.cuh).
#define FSI_LAUNCH_RO
#include "fsi_gb300.h"
#define FSI_BATCH_STEP_STORAGE FSI_STORAGE_F16
#define FSI_BATCH_PERSIST_NAME batch_persist_launch_f16
#include "batch_persistent.cuh"
