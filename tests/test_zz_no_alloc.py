"""wf_neighbour_list_static: the fixed-footprint neighbour search.

Callers that cannot allocate device memory (code inside a memory pool owned
by another library, a plugin host that forbids device allocations, a
real-time loop) pass their own input and output buffers; the search's working
memory is a fixed device array inside the library.  This checks, through the
C ABI, that three calls in a row — two on the default stream, one on a
stream of the caller's — give exactly the neighbour rows of the domain's own
rebuild (integer output: the tolerance is equality) without taking device
memory (free memory unchanged across each call after the first), that rows
with more than 100 neighbours are cut at their 100 smallest keys, and that
sizes beyond the fixed maximum — including a cell grid whose cell count
overflows 32 bits — are refused with a clear error.  The file is collected
last so a run that stops at the first failure has already run every other
test.
"""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 262144


def _cell_grid(x, h, cellfac=2.0):
    """CellInitiate (Neighbour.cpp:10-139) for a domain without DomMax/DomMin overrides."""
    blpf = [float(v) for v in x.min(axis=0)]
    trpr = [float(v) for v in x.max(axis=0)]
    hmax = float(h.max())
    no, cs = [], []
    for d in range(3):
        trpr[d] += hmax / 2
        blpf[d] -= hmax / 2
        t = (trpr[d] - blpf[d]) / (cellfac * hmax)
        no.append(int(math.ceil(t)) if (math.ceil(t) - t) < hmax / 10.0 else int(math.floor(t)))
    for d in range(3):
        cs.append((trpr[d] - blpf[d]) / no[d])
    return blpf, cs, no


def _bind(lib):
    fn = lib.wf_neighbour_list_static
    P = ctypes.c_void_p
    fn.argtypes = [P, P, P, P, ctypes.c_int64, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                   ctypes.POINTER(ctypes.c_int32), ctypes.c_double, P, P, P]
    fn.restype = ctypes.c_int
    lib.wf_last_error.restype = ctypes.c_char_p
    return fn


def test_static_search_matches_domain_rebuild_on_three_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import weldform_gb300 as wf
    from weldform_gb300 import configs

    d = wf.Domain()
    case = configs.cylinder_upsetting(d, R=0.004, L=0.010, dx=0.0004)
    x = d.get_array("x")
    h = d.get_array("h")
    d.prepare(case.dt)
    d.neighbour_search()
    off, idx = d.neighbours()
    d.close()
    n = case.n
    assert n <= MAX_N

    lib = wf.load_library()
    fn = _bind(lib)
    dev = torch.device("cuda:0")
    X = [torch.tensor(np.ascontiguousarray(x[:, k]), dtype=torch.float64, device=dev) for k in range(3)]
    H = torch.tensor(h, dtype=torch.float64, device=dev)
    blpf, cs, no = _cell_grid(x, h)
    cb = (ctypes.c_double * 3)(*blpf)
    cc = (ctypes.c_double * 3)(*cs)
    cn = (ctypes.c_int32 * 3)(*no)
    results = []
    side = torch.cuda.Stream(device=dev)
    for call in range(3):
        rl = torch.full((n,), -7, dtype=torch.int32, device=dev)
        nb = torch.full((100 * n,), -7, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(dev)[0]
        # the first two on the default stream, the third on a caller's stream
        st = ctypes.c_void_p(side.cuda_stream) if call == 2 else None
        rc = fn(X[0].data_ptr(), X[1].data_ptr(), X[2].data_ptr(), H.data_ptr(), n, cb, cc, cn, 2.0,
                rl.data_ptr(), nb.data_ptr(), st)
        assert rc == 0, lib.wf_last_error()
        torch.cuda.synchronize()
        if call > 0:  # after the first call (module load), no call takes device memory
            assert torch.cuda.mem_get_info(dev)[0] == free0
        rl_h = rl.cpu().numpy()
        nb_h = nb.cpu().numpy().reshape(100, n)
        assert (rl_h >= 0).all() and (rl_h <= 100).all()
        o = np.zeros(n + 1, dtype=np.int64)
        o[1:] = np.cumsum(rl_h)
        ix = np.concatenate([nb_h[: rl_h[i], i] for i in range(n)]).astype(np.int32)
        results.append((o, ix))
    for o, ix in results:
        assert np.array_equal(o, off)
        assert np.array_equal(ix, idx)


def test_static_search_refuses_sizes_beyond_its_maximum():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import weldform_gb300 as wf
    lib = wf.load_library()
    fn = _bind(lib)
    t = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    r = torch.zeros(8, dtype=torch.int32, device="cuda:0")
    cb = (ctypes.c_double * 3)(0, 0, 0)
    cc = (ctypes.c_double * 3)(1, 1, 1)
    cn = (ctypes.c_int32 * 3)(4, 4, 4)
    rc = fn(t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(), MAX_N + 1, cb, cc, cn, 2.0, r.data_ptr(),
            r.data_ptr(), None)
    assert rc == 1
    assert b"262144" in lib.wf_last_error()
    cn2 = (ctypes.c_int32 * 3)(2048, 2048, 2)
    rc = fn(t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(), 8, cb, cc, cn2, 2.0, r.data_ptr(), r.data_ptr(),
            None)
    assert rc == 1
    assert b"cells" in lib.wf_last_error()
    # three counts near 2^31: their product overflows 64-bit arithmetic too
    big = 2 ** 31 - 1
    cn3 = (ctypes.c_int32 * 3)(big, big, big)
    rc = fn(t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(), 8, cb, cc, cn3, 2.0, r.data_ptr(), r.data_ptr(),
            None)
    assert rc == 1
    assert b"cells" in lib.wf_last_error()


def _cut_rows_cpu(x, h, cellfac, keep=100):
    """Rows of all pairs passing CheckRadius (the same IEEE operations as the
    library: ((dx^2 + dy^2) + dz^2), sqrt, / ((hi + hj) / 2)), each kept at
    its `keep` smallest canonical keys (j - i - 1 as unsigned)."""
    n = len(x)
    rows, lens = [], []
    for i in range(n):
        d = x[i] - x
        r = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
        ok = r / ((h[i] + h) / 2.0) <= cellfac
        ok[i] = False
        j = np.nonzero(ok)[0]
        key = (j - i - 1).astype(np.int64) % (2 ** 32)
        j = j[np.argsort(key, kind="stable")]
        lens.append(len(j) if len(j) <= keep else keep + 1)
        rows.append(j[:keep])
    return rows, lens


def test_static_search_cuts_dense_rows_at_their_smallest_keys():
    """A cubic lattice with h = 2.5 spacings (pair radius 5 spacings: ~500
    neighbours per interior particle), one cell spanning the domain so every
    pair is a candidate: each cut row holds its 100 smallest keys and has
    length 101; rows that fit are complete.  Two calls agree."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import weldform_gb300 as wf
    s = 1e-3
    g = np.arange(8) * s
    x = np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(-1, 3)
    x = x + np.random.default_rng(3).uniform(-1e-3, 1e-3, x.shape) * s
    n = len(x)
    h = np.full(n, 2.5 * s)
    want_rows, want_len = _cut_rows_cpu(x, h, 2.0)
    assert max(want_len) == 101 and min(want_len) < 101
    lib = wf.load_library()
    fn = _bind(lib)
    dev = torch.device("cuda:0")
    X = [torch.tensor(np.ascontiguousarray(x[:, k]), dtype=torch.float64, device=dev) for k in range(3)]
    H = torch.tensor(h, dtype=torch.float64, device=dev)
    lo = x.min(axis=0) - 1.5 * s
    cb = (ctypes.c_double * 3)(*lo)
    cc = (ctypes.c_double * 3)(*(np.full(3, 11.0 * s)))
    cn = (ctypes.c_int32 * 3)(1, 1, 1)
    for call in range(2):
        rl = torch.full((n,), -7, dtype=torch.int32, device=dev)
        nb = torch.full((100 * n,), -7, dtype=torch.int32, device=dev)
        rc = fn(X[0].data_ptr(), X[1].data_ptr(), X[2].data_ptr(), H.data_ptr(), n, cb, cc, cn, 2.0,
                rl.data_ptr(), nb.data_ptr(), None)
        assert rc == 0, lib.wf_last_error()
        torch.cuda.synchronize()
        rl_h = rl.cpu().numpy()
        nb_h = nb.cpu().numpy().reshape(100, n)
        assert np.array_equal(rl_h, np.array(want_len))
        for i in range(n):
            k = min(rl_h[i], 100)
            assert np.array_equal(nb_h[:k, i], want_rows[i]), i
