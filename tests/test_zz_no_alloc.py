"""The allocation-free SR reduction (qmc_sr_sums_noalloc) against the
allocating entry point (qmc_logderiv_batch with S, f, e_mean).

qmc_sr_sums_noalloc exists for callers that cannot allocate device memory
(inside stream capture, memory owned by another allocator, latency-critical
loops).  It takes its scratch from a static device array.  This file is named
to be collected last; it passes alone in a fresh process and after the other
tests.  Tolerance: 1e-9 relative, as the other SR-sum tests use.
"""
import ctypes as C
import glob
import os

import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L
from tests.helpers import random_configs

pytestmark = pytest.mark.gpu


def _cudart():
    """The CUDA runtime for the test's own device buffers (the caller side
    allocates inputs and outputs; the entry point under test allocates nothing)."""
    cands = ["libcudart.so", "libcudart.so.13"] + sorted(glob.glob("/usr/local/cuda*/lib*/libcudart.so*"))
    for c in cands:
        try:
            rt = C.CDLL(c)
            rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
            rt.cudaFree.argtypes = [C.c_void_p]
            rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
            rt.cudaDeviceSynchronize.argtypes = []
            return rt
        except OSError:
            continue
    pytest.skip("no CUDA runtime library found for the test's buffers")


class DevBuf:
    def __init__(self, rt, nbytes):
        self.rt, self.ptr = rt, C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.ptr), max(nbytes, 8)) == 0

    def put(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert self.rt.cudaMemcpy(self.ptr, a.ctypes.data, a.nbytes, 1) == 0   # host -> device

    def get(self, n):
        out = np.zeros(n)
        assert self.rt.cudaMemcpy(out.ctypes.data, self.ptr, out.nbytes, 2) == 0  # device -> host
        return out

    def free(self):
        self.rt.cudaFree(self.ptr)


def sums_to_sr(sums, W, P):
    n = float(W)
    Em = sums[0] / n
    Om = sums[2:2 + P] / n
    f = sums[2 + P:2 + 2 * P] / n - Em * Om
    S = np.zeros((P, P))
    m = 2 + 2 * P
    for p in range(P):
        for q in range(p, P):
            S[p, q] = S[q, p] = sums[m] / n - Om[p] * Om[q]
            m += 1
    return S, f, Em


def test_noalloc_sr_sums_match_allocating_entry_point():
    lib = Q.load_library()
    ctx = Q.Context(0)
    spec = Q.methane_minimal()
    spec = spec.with_params(np.concatenate([spec.jas, [0.1, -0.2, 0.05, 0.3]]))
    sysh = Q.System(ctx, spec)
    rt = _cudart()
    P = sysh.num_params()
    M = 2 + 2 * P + P * (P + 1) // 2
    bufs = []
    try:
        for call, (W, seed) in enumerate([(3000, 8), (1800, 9)]):   # two calls in a row
            cfg = random_configs(spec, W, seed=seed)
            O, E, S_ref, f_ref, em_ref = sysh.logderiv_batch(cfg, sums=True)
            dE, dO, dS = DevBuf(rt, 8 * W), DevBuf(rt, 8 * W * P), DevBuf(rt, 8 * M)
            bufs += [dE, dO, dS]
            dE.put(E)
            dO.put(O)
            dS.put(np.full(M, np.nan))
            rc = lib.qmc_sr_sums_noalloc(C.cast(dE.ptr, C.POINTER(C.c_double)),
                                         C.cast(dO.ptr, C.POINTER(C.c_double)), W, P,
                                         C.cast(dS.ptr, C.POINTER(C.c_double)), None)
            assert rc == L.QMC_OK, (call, rc)
            assert rt.cudaDeviceSynchronize() == 0
            S, f, em = sums_to_sr(dS.get(M), W, P)
            np.testing.assert_allclose(S, S_ref, rtol=1e-9, atol=1e-9 * np.abs(S_ref).max())
            np.testing.assert_allclose(f, f_ref, rtol=1e-9, atol=1e-9 * np.abs(f_ref).max())
            assert abs(em - em_ref) <= 1e-9 * max(1.0, abs(em_ref))
        # sizes beyond the static scratch are rejected, not truncated
        big = lib.qmc_sr_sums_noalloc(C.cast(bufs[0].ptr, C.POINTER(C.c_double)),
                                      C.cast(bufs[1].ptr, C.POINTER(C.c_double)), 10 ** 6, P,
                                      C.cast(bufs[2].ptr, C.POINTER(C.c_double)), None)
        assert big == L.QMC_ERR_ARG
        assert lib.qmc_sr_sums_noalloc(None, None, 10, 1, None, None) == L.QMC_ERR_ARG
    finally:
        for b in bufs:
            b.free()
        sysh.close()
        ctx.close()


def test_noalloc_sr_sums_capture_and_replay():
    """After one eager call (its set-up), further eager calls leave the device's
    free memory unchanged, and the call records into a CUDA graph on a
    non-blocking stream (global capture mode): replaying that graph with new
    inputs in the same buffers gives the allocating entry point's sums."""
    lib = Q.load_library()
    ctx = Q.Context(0)
    spec = Q.methane_minimal()
    spec = spec.with_params(np.concatenate([spec.jas, [0.1, -0.2, 0.05, 0.3]]))
    sysh = Q.System(ctx, spec)
    rt = _cudart()
    rt.cudaMemGetInfo.argtypes = [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    rt.cudaStreamCreateWithFlags.argtypes = [C.POINTER(C.c_void_p), C.c_uint]
    rt.cudaStreamBeginCapture.argtypes = [C.c_void_p, C.c_int]
    rt.cudaStreamEndCapture.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    rt.cudaGraphInstantiate.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_ulonglong]
    rt.cudaGraphLaunch.argtypes = [C.c_void_p, C.c_void_p]
    rt.cudaStreamSynchronize.argtypes = [C.c_void_p]
    rt.cudaGraphExecDestroy.argtypes = [C.c_void_p]
    rt.cudaGraphDestroy.argtypes = [C.c_void_p]
    rt.cudaStreamDestroy.argtypes = [C.c_void_p]
    P = sysh.num_params()
    M = 2 + 2 * P + P * (P + 1) // 2
    W = 2048
    refs = [sysh.logderiv_batch(random_configs(spec, W, seed=s), sums=True) for s in (21, 22, 23)]
    dE, dO, dS = DevBuf(rt, 8 * W), DevBuf(rt, 8 * W * P), DevBuf(rt, 8 * M)
    dp = lambda b: C.cast(b.ptr, C.POINTER(C.c_double))

    def free_bytes():
        f, t = C.c_size_t(), C.c_size_t()
        assert rt.cudaMemGetInfo(C.byref(f), C.byref(t)) == 0
        return f.value

    stream, graph, gexec = C.c_void_p(), C.c_void_p(), C.c_void_p()
    try:
        O, E = refs[0][0], refs[0][1]
        dE.put(E)
        dO.put(O)
        assert lib.qmc_sr_sums_noalloc(dp(dE), dp(dO), W, P, dp(dS), None) == L.QMC_OK   # set-up call
        assert rt.cudaDeviceSynchronize() == 0
        free0 = free_bytes()
        for _ in range(3):
            assert lib.qmc_sr_sums_noalloc(dp(dE), dp(dO), W, P, dp(dS), None) == L.QMC_OK
        assert rt.cudaDeviceSynchronize() == 0
        assert free_bytes() == free0
        assert rt.cudaStreamCreateWithFlags(C.byref(stream), 1) == 0          # non-blocking
        assert rt.cudaStreamBeginCapture(stream, 0) == 0                      # global mode
        rc = lib.qmc_sr_sums_noalloc(dp(dE), dp(dO), W, P, dp(dS), stream)
        assert rt.cudaStreamEndCapture(stream, C.byref(graph)) == 0
        assert rc == L.QMC_OK
        assert rt.cudaGraphInstantiate(C.byref(gexec), graph, 0) == 0
        for O, E, S_ref, f_ref, em_ref in refs[1:]:
            dE.put(E)
            dO.put(O)
            dS.put(np.full(M, np.nan))
            assert rt.cudaGraphLaunch(gexec, stream) == 0
            assert rt.cudaStreamSynchronize(stream) == 0
            S, f, em = sums_to_sr(dS.get(M), W, P)
            np.testing.assert_allclose(S, S_ref, rtol=1e-9, atol=1e-9 * np.abs(S_ref).max())
            np.testing.assert_allclose(f, f_ref, rtol=1e-9, atol=1e-9 * np.abs(f_ref).max())
            assert abs(em - em_ref) <= 1e-9 * max(1.0, abs(em_ref))
    finally:
        if gexec.value:
            rt.cudaGraphExecDestroy(gexec)
        if graph.value:
            rt.cudaGraphDestroy(graph)
        if stream.value:
            rt.cudaStreamDestroy(stream)
        for b in (dE, dO, dS):
            b.free()
        sysh.close()
        ctx.close()
