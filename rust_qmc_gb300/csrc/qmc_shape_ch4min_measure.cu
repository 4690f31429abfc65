// qmc_shape_ch4min_measure.cu -- initialisation and measurement kernels for the ShapeCH4Min system shape.
#include "qmc_walker_kernels.cuh"

namespace qmc {
QMC_DEFINE_SHAPE_MEASURE(ch4min, ShapeCH4Min)
}  // namespace qmc
