"""cnn_fit_csr_noalloc: the fit for callers that cannot allocate device memory.

Some callers may not allocate GPU memory while they run -- a serving loop
with a memory budget fixed at start-up, a plug-in inside a framework whose
caching allocator already holds the free memory, a latency-critical loop
that cannot afford the device-wide synchronisation cudaMalloc/cudaFree may
cause.  This entry point takes only the caller's inputs and outputs and uses
a fixed scratch block compiled into the library.  Its results must be
identical to the allocating path (cnn_set_neighbours + cnn_fit) on the same
graph, call after call, since every call reuses the same scratch.

The file is named to be collected last, and it creates everything it needs,
so it passes both alone in a fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from commonnnclustering_gb300 import _abi
    return torch, _abi


def graph(_abi, x, radius_cutoff):
    ctx = _abi.Context(0)
    ctx.set_points(x)
    ctx.build_neighbours(radius_cutoff)
    off, idx = ctx.get_neighbours(x.shape[0])
    ctx.close()
    return off, idx


def allocating_fit(_abi, off, idx, sc, nm, cs, consider, labels):
    ctx = _abi.Context(0)
    ctx.set_neighbours(off, idx)
    lab, con = labels.copy(), consider.copy()
    ctx.fit(sc, nm, cs, con, lab)
    ctx.close()
    return lab, con


def noalloc_fit(torch, _abi, off, idx, sc, nm, cs, consider, labels):
    lib = _abi.load()
    dev = torch.device("cuda", 0)
    d_off = torch.from_numpy(off).to(dev)
    d_idx = torch.from_numpy(idx).to(dev)
    d_con = torch.from_numpy(consider.copy()).to(dev)
    d_lab = torch.from_numpy(labels.copy()).to(dev)
    stream = torch.cuda.current_stream(dev)
    st = lib.cnn_fit_csr_noalloc(ctypes.c_void_p(d_off.data_ptr()), ctypes.c_void_p(d_idx.data_ptr()),
                                 off.shape[0] - 1, sc, nm, cs, ctypes.c_void_p(d_con.data_ptr()),
                                 ctypes.c_void_p(d_lab.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert st == 0, st
    torch.cuda.synchronize(dev)
    return d_lab.cpu().numpy(), d_con.cpu().numpy()


def test_noalloc_matches_allocating_path_on_consecutive_calls(env):
    torch, _abi = env
    from commonnnclustering_gb300 import workloads
    rng = np.random.default_rng(21)
    cases = []
    x1 = workloads.md3d(n=40000, seed=4, centre_spread=2.0)
    cases.append((x1, 0.12 ** 2, 7, 6, 1, None))
    x2 = workloads.blobs2d(n=5000, seed=2)
    cons = (rng.random(5000) < 0.7).astype(np.uint8)
    cases.append((x2, 0.3 ** 2, 7, 6, 5, cons))
    cases.append((x1, 0.12 ** 2, 22, 21, 1, None))  # same graph again, other cutoffs
    for x, r2, sc, nm, cs, consider in cases:
        off, idx = graph(_abi, x, r2)
        n = x.shape[0]
        if consider is None:
            consider = np.ones(n, dtype=np.uint8)
        labels = np.where(consider == 0, 9, 0).astype(np.int64)
        want_l, want_c = allocating_fit(_abi, off, idx, sc, nm, cs, consider, labels)
        got_l, got_c = noalloc_fit(torch, _abi, off, idx, sc, nm, cs, consider, labels)
        assert np.array_equal(got_l, want_l)
        assert np.array_equal(got_c, want_c)
        assert len(set(got_l.tolist()) - {0, 9}) > 1


def test_noalloc_leaves_outputs_untouched_for_an_invalid_graph(env):
    """A bad graph is caught on the GPU before it is read: an index in
    [n, CNN_NOALLOC_MAX_POINTS) (which would otherwise read stale scratch),
    a row out of order, or decreasing offsets leave labels and consider as
    they were; the next valid call is fitted as usual."""
    torch, _abi = env
    from commonnnclustering_gb300 import workloads
    x = workloads.blobs2d(n=3000, seed=5)
    off, idx = graph(_abi, x, 0.3 ** 2)
    n = x.shape[0]
    consider = np.ones(n, dtype=np.uint8)
    labels = np.full(n, 7, dtype=np.int64)
    row = int(np.argmax(np.diff(off)))          # a long row
    s, e = int(off[row]), int(off[row + 1])
    bad_index = idx.copy()
    bad_index[e - 1] = n + 5                     # beyond the graph, inside the scratch block
    bad_order = idx.copy()
    bad_order[s], bad_order[s + 1] = bad_order[s + 1], bad_order[s]
    bad_off = off.copy()
    bad_off[row + 1] = bad_off[row] - 1          # a decreasing offset
    for o, i in ((off, bad_index), (off, bad_order), (bad_off, idx)):
        got_l, got_c = noalloc_fit(torch, _abi, o, i, 7, 6, 1, consider, labels)
        assert np.array_equal(got_l, labels)
        assert np.array_equal(got_c, consider)
    want_l, want_c = allocating_fit(_abi, off, idx, 7, 6, 1, consider, labels)
    got_l, got_c = noalloc_fit(torch, _abi, off, idx, 7, 6, 1, consider, labels)
    assert np.array_equal(got_l, want_l) and np.array_equal(got_c, want_c)
    assert not got_c.any()


def test_noalloc_rejects_more_points_than_its_scratch_holds(env):
    torch, _abi = env
    lib = _abi.load()
    dev = torch.device("cuda", 0)
    small = torch.zeros(8, dtype=torch.int64, device=dev)
    st = lib.cnn_fit_csr_noalloc(ctypes.c_void_p(small.data_ptr()), ctypes.c_void_p(small.data_ptr()),
                                 65536 + 1, 2, 1, 1, ctypes.c_void_p(small.data_ptr()),
                                 ctypes.c_void_p(small.data_ptr()), None)
    assert st == 1  # CNN_ERR_INVALID_ARG, nothing queued
    assert not torch.any(small).item()
