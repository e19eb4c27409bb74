"""The allocation-free APC/ASC entry point (covgpu_correct_noalloc), called
through the C-ABI, against the FP64 oracle's corr_CalculateCOVCorrected
restatement (orc_cov_corrected) and the allocating entry point
(covgpu_correct), two calls in a row.

Callers that cannot allocate device memory (code inside a stream capture,
pooled-memory hosts, real-time callers) pass device buffers they own; the
entry point keeps its scratch in a fixed device array.  This file also
captures the call into a CUDA graph and replays it, with no change of the
device memory in use, and checks in-place use and the NaN report.  Needs a
GB300; device buffers for the test itself come from torch.
"""
import ctypes as C

import numpy as np
import pytest

from parity_tol import stat_close

pytestmark = pytest.mark.gpu


def scores(covgpu, N, L, seed, stat):
    s = covgpu.Synth(N, L, 1.5, L // 6, 1, 1, L // 6, 0.1, seed=seed, tree_kind=1)
    w = covgpu.weights_pb(s.ax)
    e = covgpu.Engine(N, L)
    e.set_weights(w)
    e.set_alignment(0, s.ax)
    e.score([stat])
    cov = e.get_cov(0, 0)
    return e, cov


def noalloc(covgpu):
    lib = covgpu.lib()
    lib.covgpu_correct_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    lib.covgpu_correct_noalloc.restype = C.c_int
    return lib


def reference_correct(covgpu, e, cov, actype):
    lib = covgpu.lib()
    lib.covgpu_correct.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L = cov.shape[0]
    cin = np.ascontiguousarray(cov)
    out = np.zeros(L * L)
    mm = np.zeros(2)
    st = lib.covgpu_correct(e.h, cin.ctypes.data, actype, out.ctypes.data, mm.ctypes.data)
    assert st == 0, lib.covgpu_errmsg(e.h)
    return out.reshape(L, L), mm


def oracle_correct(oracle, cov, actype):
    L = cov.shape[0]
    out = np.ascontiguousarray(cov, dtype=np.float64).ravel().copy()
    mm = np.zeros(2)
    assert oracle.lib().orc_cov_corrected(actype, L, out, mm) == 0
    return out.reshape(L, L), mm


def check(got, mm, ref, ref_mm):
    L = got.shape[0]
    off = ~np.eye(L, dtype=bool)
    ok, rel, small = stat_close(got[off], ref[off])
    assert ok, (rel, small)
    assert np.all(np.isneginf(np.diag(got)))
    assert np.allclose(mm, ref_mm, rtol=1e-5, atol=1e-8 * np.max(np.abs(ref[off])))


def test_noalloc_matches_oracle_and_allocating_entry_point(covgpu, oracle):
    torch = pytest.importorskip("torch")
    lib = noalloc(covgpu)
    cases = [(120, 90, 3, "GT", 0), (80, 130, 5, "MI", 1)]   # APC, then ASC on another matrix
    for N, L, seed, stat, actype in cases:
        e, cov = scores(covgpu, N, L, seed, stat)
        ref, ref_mm = oracle_correct(oracle, cov, actype)
        lib_ref, lib_mm = reference_correct(covgpu, e, cov, actype)
        d_cov = torch.tensor(cov, dtype=torch.float64, device="cuda")
        d_out = torch.zeros((L, L), dtype=torch.float64, device="cuda")
        d_mm = torch.zeros(2, dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream()
        st = lib.covgpu_correct_noalloc(d_cov.data_ptr(), d_out.data_ptr(), L, actype, d_mm.data_ptr(),
                                        stream.cuda_stream)
        assert st == 0
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        mm = d_mm.cpu().numpy()
        check(got, mm, ref, ref_mm)
        check(got, mm, lib_ref, lib_mm)
        # in place: the output written over the input
        st = lib.covgpu_correct_noalloc(d_cov.data_ptr(), d_cov.data_ptr(), L, actype, d_mm.data_ptr(),
                                        stream.cuda_stream)
        assert st == 0
        torch.cuda.synchronize()
        check(d_cov.cpu().numpy(), d_mm.cpu().numpy(), ref, ref_mm)
        e.close()


def test_noalloc_in_a_cuda_graph(covgpu, oracle):
    """A warm call, then the call captured on a side stream into a CUDA graph
    and replayed on new data: the result matches the oracle and the device
    memory in use does not change across the replay."""
    torch = pytest.importorskip("torch")
    lib = noalloc(covgpu)
    N, L = 100, 110
    e, cov = scores(covgpu, N, L, 8, "GT")
    e2, cov2 = scores(covgpu, N, L, 9, "GT")
    d_cov = torch.tensor(cov, dtype=torch.float64, device="cuda")
    d_out = torch.zeros((L, L), dtype=torch.float64, device="cuda")
    d_mm = torch.zeros(2, dtype=torch.float64, device="cuda")
    # the warm call (looks up the scratch address, loads the kernels)
    assert lib.covgpu_correct_noalloc(d_cov.data_ptr(), d_out.data_ptr(), L, 0, d_mm.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            st = lib.covgpu_correct_noalloc(d_cov.data_ptr(), d_out.data_ptr(), L, 0, d_mm.data_ptr(),
                                            torch.cuda.current_stream().cuda_stream)
    assert st == 0
    torch.cuda.synchronize()
    d_cov.copy_(torch.tensor(cov2, dtype=torch.float64))
    d_out.zero_()
    torch.cuda.synchronize()
    used0, free0 = torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0]
    g.replay()
    torch.cuda.synchronize()
    assert torch.cuda.memory_allocated() == used0
    assert torch.cuda.mem_get_info()[0] == free0
    ref, ref_mm = oracle_correct(oracle, cov2, 0)
    check(d_out.cpu().numpy(), d_mm.cpu().numpy(), ref, ref_mm)
    e.close()
    e2.close()


def test_noalloc_reports_nan(covgpu):
    """A NaN score makes corrected scores NaN (the reference's "bad
    covariation" error): the call reports it as a NaN min/max."""
    torch = pytest.importorskip("torch")
    lib = noalloc(covgpu)
    L = 40
    cov = np.random.default_rng(1).uniform(0, 5, (L, L))
    cov = (cov + cov.T) / 2
    cov[3, 7] = cov[7, 3] = np.nan
    d_cov = torch.tensor(cov, dtype=torch.float64, device="cuda")
    d_out = torch.zeros((L, L), dtype=torch.float64, device="cuda")
    d_mm = torch.zeros(2, dtype=torch.float64, device="cuda")
    assert lib.covgpu_correct_noalloc(d_cov.data_ptr(), d_out.data_ptr(), L, 0, d_mm.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    assert np.all(np.isnan(d_mm.cpu().numpy()))
    # the next call on good data clears the report
    cov[3, 7] = cov[7, 3] = 1.0
    d_cov.copy_(torch.tensor(cov, dtype=torch.float64))
    assert lib.covgpu_correct_noalloc(d_cov.data_ptr(), d_out.data_ptr(), L, 0, d_mm.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    assert np.all(np.isfinite(d_mm.cpu().numpy()))


def test_noalloc_rejects_sizes_beyond_its_limit(covgpu):
    lib = noalloc(covgpu)
    # rejected before any device work: the pointers are never dereferenced
    assert lib.covgpu_correct_noalloc(C.c_void_p(16), C.c_void_p(16), 16385, 0, C.c_void_p(16), None) == 11
    assert lib.covgpu_correct_noalloc(C.c_void_p(16), C.c_void_p(16), 1, 0, C.c_void_p(16), None) == 11
    assert lib.covgpu_correct_noalloc(C.c_void_p(16), C.c_void_p(16), 100, 7, C.c_void_p(16), None) == 11
