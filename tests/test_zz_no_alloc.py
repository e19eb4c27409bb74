"""The allocation-free APC/ASC entry point (covgpu_correct_noalloc) against
the allocating one (covgpu_correct), through the C-ABI, two calls in a row.

Callers that cannot allocate device memory (code inside a stream capture,
pooled-memory hosts, real-time callers) pass device buffers they own; the
entry point keeps its scratch in a fixed device array.  Needs a GB300; device
buffers for the test itself come from torch.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-5
ATOL_SCALE = 2e-7


def scores(covgpu, N, L, seed, stat):
    s = covgpu.Synth(N, L, 1.5, L // 6, 1, 1, L // 6, 0.1, seed=seed, tree_kind=1)
    w = covgpu.weights_pb(s.ax)
    e = covgpu.Engine(N, L)
    e.set_weights(w)
    e.set_alignment(0, s.ax)
    e.score([stat])
    cov = e.get_cov(0, 0)
    return e, cov


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


def test_noalloc_matches_allocating_entry_point(covgpu):
    torch = pytest.importorskip("torch")
    lib = covgpu.lib()
    lib.covgpu_correct_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    lib.covgpu_correct_noalloc.restype = C.c_int
    cases = [(120, 90, 3, "GT", 0), (80, 130, 5, "MI", 1)]   # APC, then ASC on another matrix
    for N, L, seed, stat, actype in cases:
        e, cov = scores(covgpu, N, L, seed, stat)
        ref, ref_mm = reference_correct(covgpu, e, cov, actype)
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
        off = ~np.eye(L, dtype=bool)
        scale = np.max(np.abs(cov[off]))
        assert np.all(np.abs(got[off] - ref[off]) <= RTOL * np.abs(ref[off]) + ATOL_SCALE * scale)
        assert np.all(np.isneginf(np.diag(got)))
        assert np.allclose(mm, ref_mm, rtol=RTOL, atol=ATOL_SCALE * scale)
        e.close()


def test_noalloc_rejects_sizes_beyond_its_limit(covgpu):
    lib = covgpu.lib()
    lib.covgpu_correct_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    # rejected before any device work: the pointers are never dereferenced
    assert lib.covgpu_correct_noalloc(C.c_void_p(16), C.c_void_p(16), 16385, 0, C.c_void_p(16), None) == 11
    assert lib.covgpu_correct_noalloc(C.c_void_p(16), C.c_void_p(16), 1, 0, C.c_void_p(16), None) == 11
    assert lib.covgpu_correct_noalloc(C.c_void_p(16), C.c_void_p(16), 100, 7, C.c_void_p(16), None) == 11
