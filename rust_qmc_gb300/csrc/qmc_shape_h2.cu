// qmc_shape_h2.cu -- all kernels for the ShapeH2 system shape.
#include "qmc_walker_kernels.cuh"

namespace qmc {
QMC_DEFINE_SHAPE_MEASURE(h2, ShapeH2)
QMC_DEFINE_SHAPE_ONE(h2, ShapeH2)
QMC_DEFINE_SHAPE_ALL(h2, ShapeH2)
QMC_DEFINE_SHAPE_BATCH_SWEEP(h2, ShapeH2)
QMC_DEFINE_SHAPE_BATCH_MEASURE(h2, ShapeH2)
}  // namespace qmc
