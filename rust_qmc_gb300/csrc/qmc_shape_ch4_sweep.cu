// qmc_shape_ch4_sweep.cu -- single-electron sweep kernels for the ShapeCH4 system shape.
#include "qmc_walker_kernels.cuh"

namespace qmc {
QMC_DEFINE_SHAPE_ONE(ch4, ShapeCH4)
}  // namespace qmc
