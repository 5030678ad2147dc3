// Batched step kernels of the 64^3 size class.
#include "ffs_batch_class.cuh"
FFS_DEFINE_BATCH_CLASS(64, 3)
