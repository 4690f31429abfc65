// qmc_shape_ch4min_sweep.cu -- single-electron sweep kernels for the ShapeCH4Min system shape.
#include "qmc_walker_kernels.cuh"

namespace qmc {
QMC_DEFINE_SHAPE_ONE(ch4min, ShapeCH4Min)
}  // namespace qmc
