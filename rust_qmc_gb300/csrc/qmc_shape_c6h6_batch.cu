// qmc_shape_c6h6_batch.cu -- batched kernels for the c6h6 shape.
#include "qmc_warp_kernels.cuh"

namespace qmc {
using Ops_c6h6 = WarpShapeOps<42, 21, 12>;
int shape_batch_sweep_c6h6(const BatchClass& bc, int mk, const BatchCtl* ctl, cudaStream_t st, int* occ) {
    return Ops_c6h6::batch_sweep(bc, mk, ctl, st, occ);
}
int shape_batch_measure_c6h6(const BatchClass& bc, cudaStream_t st, int* occ) {
    return Ops_c6h6::batch_measure(bc, st, occ);
}
int shape_batch_tables_c6h6(const HostSys& hs, int prec, BatchRec& r) { return Ops_c6h6::batch_tables(hs, prec, r); }
int shape_batch_width_c6h6() { return Ops_c6h6::BTW; }
}  // namespace qmc
