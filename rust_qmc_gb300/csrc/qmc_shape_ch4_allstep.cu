// qmc_shape_ch4_allstep.cu -- all-electron step kernels for the ShapeCH4 system shape.
#include "qmc_walker_kernels.cuh"

namespace qmc {
QMC_DEFINE_SHAPE_ALL(ch4, ShapeCH4)
}  // namespace qmc
