// Batched step kernels of the 32^3 size class.
#include "ffs_batch_class.cuh"
FFS_DEFINE_BATCH_CLASS(32, 1)
