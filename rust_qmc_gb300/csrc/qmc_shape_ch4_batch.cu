// qmc_shape_ch4_batch.cu -- batched kernels for the ShapeCH4 system shape.
#include "qmc_walker_kernels.cuh"

namespace qmc {
QMC_DEFINE_SHAPE_BATCH_SWEEP(ch4, ShapeCH4)
QMC_DEFINE_SHAPE_BATCH_MEASURE(ch4, ShapeCH4)
}  // namespace qmc
