// Batched step kernels of the 128^3 size class.
#include "ffs_batch_class.cuh"
FFS_DEFINE_BATCH_CLASS(128, 5)
