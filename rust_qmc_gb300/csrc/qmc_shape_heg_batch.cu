// qmc_shape_heg_batch.cu -- batched kernels for the heg shape.
#include "qmc_heg_kernels.cuh"

namespace qmc {
using Ops_heg = HegShapeOps<54, 27>;
int shape_batch_sweep_heg(const BatchClass& bc, int mk, const BatchCtl* ctl, cudaStream_t st, int* occ) {
    return Ops_heg::batch_sweep(bc, mk, ctl, st, occ);
}
int shape_batch_measure_heg(const BatchClass& bc, cudaStream_t st, int* occ) {
    return Ops_heg::batch_measure(bc, st, occ);
}
int shape_batch_tables_heg(const HostSys& hs, int prec, BatchRec& r) { return Ops_heg::batch_tables(hs, prec, r); }
int shape_batch_width_heg() { return Ops_heg::WPB; }
}  // namespace qmc
