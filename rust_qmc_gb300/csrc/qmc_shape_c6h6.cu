// qmc_shape_c6h6.cu -- warp-per-walker kernels for the benzene shape
// (42 electrons, 21 + 21, 12 nuclei, up to 96 Gaussian AOs, Jastrow3 form).
#include "qmc_warp_kernels.cuh"

namespace qmc {
using C6H6Ops = WarpShapeOps<42, 21, 12>;
int shape_init_c6h6(const HostSys& hs, DevWalkers& dw, uint64_t seed, cudaStream_t st) {
    return C6H6Ops::init(hs, dw, seed, st);
}
int shape_measure_c6h6(const HostSys& hs, DevWalkers& dw, int cp, bool ws, const MeasureOut& out, cudaStream_t st) {
    return C6H6Ops::measure(hs, dw, cp, ws, out, st);
}
int shape_sweep_one_c6h6(const HostSys& hs, DevWalkers& dw, int mk, int n, uint64_t s0, double step, double tau,
                         double maxd, uint64_t seed, cudaStream_t st) {
    return C6H6Ops::sweep(hs, dw, mk, n, s0, step, tau, maxd, seed, st);
}
int shape_step_all_c6h6(const HostSys&, DevWalkers&, int, int, uint64_t, double, uint64_t, cudaStream_t, double*) {
    return 7;   // all-electron moves are not compiled for the benzene shape
}
int shape_nmax_c6h6() { return C6H6Ops::NM; }
}  // namespace qmc
