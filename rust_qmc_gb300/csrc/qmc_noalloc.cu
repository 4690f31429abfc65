// qmc_noalloc.cu -- allocation-free variant of the SR walker-sum reduction.
//
// qmc_sr_sums_noalloc runs the same two reduction kernels as
// qmc_logderiv_batch's S/f path (k_sr_partials + k_sum_partials via
// launch_sr_sums), but takes its block-partial scratch from a statically
// allocated device array instead of memory obtained from cudaMalloc.  It is
// meant for callers that must not allocate device memory: code running
// between cudaStreamBeginCapture and cudaStreamEndCapture, hosts whose device
// memory is owned by another framework's allocator, and latency-critical
// loops that cannot afford the implicit device synchronisation of cudaFree.
#include <cstdio>
#include <mutex>
#include <cuda_runtime.h>
#include "../../include/qmc.h"
#include "qmc_internal.h"

namespace {

// 65 536 doubles = 512 KiB, held by every GPU that loads the library until
// the process exits.
constexpr int kScratchDoubles = 65536;
__device__ __align__(256) double g_sr_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of g_sr_scratch on the current device.  In host code the
// symbol's name is only a host-side stand-in, so the address is looked up
// once per device (with that device current) and cached.
int scratch_address(int device, double** out) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_sr_scratch);
        if (e != cudaSuccess || !p) {
            std::fprintf(stderr, "qmc_sr_sums_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            return QMC_ERR_CUDA;
        }
        g_scratch_addr[device] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[device];
    return QMC_OK;
}

}  // namespace

extern "C" int qmc_sr_sums_noalloc(const double* d_E, const double* d_O, int W, int P, double* d_sums,
                                   void* stream) {
    if (!d_E || !d_sums || W <= 0 || P < 0 || (P > 0 && !d_O)) return QMC_ERR_ARG;
    if (P > QMC_NOALLOC_MAX_PARAMS) {
        std::fprintf(stderr, "qmc_sr_sums_noalloc: P = %d exceeds the maximum of %d parameters\n", P,
                     QMC_NOALLOC_MAX_PARAMS);
        return QMC_ERR_ARG;
    }
    // Same blocking as launch_sr_sums: ceil(W/256) chunks, at most 1024.
    long long M = 2 + 2LL * P + (long long)P * (P + 1) / 2;
    long long nblk = (W + 255) / 256;
    if (nblk > 1024) nblk = 1024;
    if (2 * M * nblk > kScratchDoubles) {
        std::fprintf(stderr,
                     "qmc_sr_sums_noalloc: W = %d, P = %d needs %lld scratch doubles; the static scratch holds %d "
                     "(2 (2 + 2P + P(P+1)/2) ceil(W/256) must not exceed it)\n",
                     W, P, 2 * M * nblk, kScratchDoubles);
        return QMC_ERR_ARG;
    }
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) return QMC_ERR_CUDA;
    double* scratch = nullptr;
    int rc = scratch_address(device, &scratch);
    if (rc) return rc;
    // Every block-partial slot the reduction reads is written earlier in the
    // same call, so the scratch needs no clearing between calls.
    return qmc::launch_sr_sums(d_E, d_O, W, P, d_sums, scratch, kScratchDoubles,
                               static_cast<cudaStream_t>(stream));
}
