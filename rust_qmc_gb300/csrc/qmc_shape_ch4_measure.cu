// qmc_shape_ch4_measure.cu -- initialisation and measurement kernels for the ShapeCH4 system shape.
#include "qmc_walker_kernels.cuh"

namespace qmc {
QMC_DEFINE_SHAPE_MEASURE(ch4, ShapeCH4)
}  // namespace qmc
