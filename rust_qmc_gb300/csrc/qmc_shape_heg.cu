// qmc_shape_heg.cu -- warp-per-walker kernels of the 54-electron periodic
// electron gas (27 + 27 plane waves).
#include "qmc_heg_kernels.cuh"

namespace qmc {
using HegOps = HegShapeOps<54, 27>;
int shape_init_heg(const HostSys& hs, DevWalkers& dw, uint64_t seed, cudaStream_t st) {
    return HegOps::init(hs, dw, seed, st);
}
int shape_measure_heg(const HostSys& hs, DevWalkers& dw, int cp, bool ws, const MeasureOut& out, cudaStream_t st) {
    return HegOps::measure(hs, dw, cp, ws, out, st);
}
int shape_sweep_one_heg(const HostSys& hs, DevWalkers& dw, int mk, int n, uint64_t s0, double step, double tau,
                        double maxd, uint64_t seed, cudaStream_t st) {
    return HegOps::sweep(hs, dw, mk, n, s0, step, tau, maxd, seed, st);
}
int shape_step_all_heg(const HostSys&, DevWalkers&, int, int, uint64_t, double, uint64_t, cudaStream_t, double*) {
    return 7;   // all-electron moves are not compiled for the electron gas
}
int shape_nmax_heg() { return HegOps::NM; }
}  // namespace qmc
