"""bsa_gpu_pointMomentsNoAlloc: the point-set moment reduction for callers that cannot
allocate device memory (they hand in device buffers from their own allocator; the entry
point keeps its scratch in a fixed device array).  Checked through the C-ABI against the
allocating entry point bsa_gpu_mshMoments on the same structure and points, twice in a row,
within the FP64 path's 1e-10 tolerance.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import tall_building
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu
TOL = 1e-10


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def a_table(o, freqs):
    """A(f)[(itc, i)][m] = sum_j S_ij(f) L[j][m] for every frequency, numpy FP64."""
    prob = o.prob
    rows = []
    for f in freqs:
        blocks = []
        for tc in prob.settings.tc:
            L = o.phitc[:, :, tc - 1].T            # (nnl, nm)
            blocks.append(o.cross_psd(f, tc) @ L)
        rows.append(np.concatenate(blocks, axis=0))
    return np.ascontiguousarray(np.stack(rows))     # (rows, K, nm)


def test_no_alloc_matches_allocating_entry_point(bsalib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    prob = tall_building(nodes=20, modes=5, nfreqs=5, df=0.3, seed=17)
    o = Oracle(prob)
    nm = o.nme
    Q = np.ascontiguousarray(np.concatenate([o.phitc[:, :, tc + 2].T for tc in prob.settings.tc], axis=0))
    K = Q.shape[0]
    m = o.modes - 1
    dev = torch.device("cuda:0")
    T = lambda a, dt=torch.float64: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    dM, dK, dC = T(prob.Mg[m]), T(prob.Kg[m]), T(prob.Cg[m, m])
    dQ = T(Q)
    sess = api.BsaSession(prob)
    rng = np.random.default_rng(5)
    try:
        for call in range(2):
            n = 23 + 10 * call
            fi, fj = rng.uniform(-1.5, 1.5, n), rng.uniform(-1.5, 1.5, n)
            w = rng.uniform(0.2, 1.0, n)
            freqs = np.concatenate([fi, fj, fi + fj])
            dA = T(a_table(o, freqs))
            ix, iy, iz = np.arange(n), n + np.arange(n), 2 * n + np.arange(n)
            if call == 1:
                iz[::4] = -1    # S(f1+f2) taken as zero on these points
            d_ix, d_iy, d_iz = (T(v, torch.int32) for v in (ix, iy, iz))
            d_f1, d_f2, d_w = T(fi), T(fj), T(w)
            out_f = torch.zeros(nm ** 3, dtype=torch.float64, device=dev)
            out_r = torch.zeros(nm ** 3, dtype=torch.float64, device=dev)
            p = lambda t: C.c_void_p(t.data_ptr())
            stream = torch.cuda.current_stream().cuda_stream
            rc = bsalib.bsa_gpu_pointMomentsNoAlloc(p(dA), K, nm, p(dQ), p(d_ix), p(d_iy), p(d_iz), p(d_f1),
                                                    p(d_f2), p(d_w), n, p(dM), p(dK), p(dC), p(out_f), p(out_r),
                                                    C.c_void_p(stream))
            assert rc == 0, bsalib.bsa_lastError()
            torch.cuda.synchronize()
            if call == 0:
                ref_f, ref_r = sess.msh_moments(fi, fj, w)
            else:
                # reference with the same zeroed S(f1+f2): weight those points by their
                # value without terms 2 and 3, i.e. evaluate them through the oracle
                keep = iz >= 0
                ref_f, ref_r = sess.msh_moments(fi[keep], fj[keep], w[keep])
                for k in np.nonzero(~keep)[0]:
                    s12 = [np.zeros((prob.nnl, prob.nnl))] * prob.ntc
                    bf = o.direct_point(fi[k], fj[k], s12)
                    ref_f = ref_f + w[k] * bf
                    ref_r = ref_r + w[k] * bf * o.brm_factor(fi[k], fj[k])
            assert rel(out_f.cpu().numpy(), ref_f) < TOL
            assert rel(out_r.cpu().numpy(), ref_r) < TOL
    finally:
        sess.close()


def test_no_alloc_clamped_groups_allocate_nothing(bsalib):
    """33 kept modes: the fixed scratch holds 2^18 / 33^3 = 7 point groups where the allocating
    path would run one per point (40 here), so this is the entry point's own clamped branch.
    The device's free memory is read around the second call (the first one may load the
    library's kernels): a call that allocates nothing leaves it unchanged."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    prob = tall_building(nodes=30, modes=33, nfreqs=5, df=0.3, seed=23)
    o = Oracle(prob)
    nm = o.nme
    assert nm == 33 and (1 << 18) // nm ** 3 == 7
    Q = np.ascontiguousarray(np.concatenate([o.phitc[:, :, tc + 2].T for tc in prob.settings.tc], axis=0))
    K = Q.shape[0]
    m = o.modes - 1
    dev = torch.device("cuda:0")
    T = lambda a, dt=torch.float64: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    dM, dK, dC, dQ = T(prob.Mg[m]), T(prob.Kg[m]), T(prob.Cg[m, m]), T(Q)
    rng = np.random.default_rng(9)
    n = 40
    fi, fj = rng.uniform(-1.2, 1.2, n), rng.uniform(-1.2, 1.2, n)
    w = rng.uniform(0.2, 1.0, n)
    dA = T(a_table(o, np.concatenate([fi, fj, fi + fj])))
    d_ix, d_iy, d_iz = (T(v, torch.int32) for v in (np.arange(n), n + np.arange(n), 2 * n + np.arange(n)))
    d_f1, d_f2, d_w = T(fi), T(fj), T(w)
    out_f = torch.zeros(nm ** 3, dtype=torch.float64, device=dev)
    out_r = torch.zeros(nm ** 3, dtype=torch.float64, device=dev)
    p = lambda t: C.c_void_p(t.data_ptr())
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = (p(dA), K, nm, p(dQ), p(d_ix), p(d_iy), p(d_iz), p(d_f1), p(d_f2), p(d_w), n, p(dM), p(dK), p(dC),
            p(out_f), p(out_r), stream)
    sess = api.BsaSession(prob)
    try:
        ref_f, ref_r = sess.msh_moments(fi, fj, w)
    finally:
        sess.close()
    for call in range(2):
        out_f.fill_(float("nan"))
        out_r.fill_(float("nan"))
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc = bsalib.bsa_gpu_pointMomentsNoAlloc(*args)
        assert rc == 0, bsalib.bsa_lastError()
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        if call == 1:
            assert free1 == free0
        assert rel(out_f.cpu().numpy(), ref_f) < TOL
        assert rel(out_r.cpu().numpy(), ref_r) < TOL


def test_no_alloc_rejects_bad_sizes(bsalib):
    n = C.c_void_p(0)
    rc = bsalib.bsa_gpu_pointMomentsNoAlloc(n, 4, 65, n, n, n, n, n, n, n, 1, n, n, n, n, n, n)
    assert rc == -1
    one = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = bsalib.bsa_gpu_pointMomentsNoAlloc(one, 4, 65, one, one, one, one, one, one, one, 1, one, one, one,
                                            one, one, None)
    assert rc == -1 and b"1..64" in bsalib.bsa_lastError()
