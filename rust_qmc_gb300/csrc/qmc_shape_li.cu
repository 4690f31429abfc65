// qmc_shape_li.cu -- all kernels for the ShapeLi system shape.
#include "qmc_walker_kernels.cuh"

namespace qmc {
QMC_DEFINE_SHAPE_MEASURE(li, ShapeLi)
QMC_DEFINE_SHAPE_ONE(li, ShapeLi)
QMC_DEFINE_SHAPE_ALL(li, ShapeLi)
QMC_DEFINE_SHAPE_BATCH_SWEEP(li, ShapeLi)
QMC_DEFINE_SHAPE_BATCH_MEASURE(li, ShapeLi)
}  // namespace qmc
