// qmc_shape_ch4min_batch.cu -- batched kernels for the ShapeCH4Min system shape.
#include "qmc_walker_kernels.cuh"

namespace qmc {
QMC_DEFINE_SHAPE_BATCH_SWEEP(ch4min, ShapeCH4Min)
QMC_DEFINE_SHAPE_BATCH_MEASURE(ch4min, ShapeCH4Min)
}  // namespace qmc
