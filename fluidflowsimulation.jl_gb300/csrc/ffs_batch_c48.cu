// Batched step kernels of the 48^3 size class.
#include "ffs_batch_class.cuh"
FFS_DEFINE_BATCH_CLASS(48, 2)
