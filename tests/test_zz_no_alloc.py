"""lvg_modularity_noalloc: modularity for callers that cannot allocate device memory.

Such callers (a framework that has reserved the GPU's memory for its own
pool, a latency-critical loop that must not pay cudaMalloc's cost, a
deployment that forbids allocation after start-up) own every buffer: the test
plays that caller, allocating the inputs and the output on the device itself
(with torch), and checks the result of two calls in a row against the
allocating entry point lvg_modularity, within the FP64 tolerance used for
modularity elsewhere (1e-12 absolute; the two differ only in the order of
their FP64 atomic additions).

This file is named to be collected last.
"""
import numpy as np
import pytest

from conftest import Golden

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _dev(torch, a: np.ndarray, dt):
    return torch.from_numpy(np.ascontiguousarray(a).view(dt)).to("cuda:0")


def test_noalloc_matches_allocating_entry_point_twice(cuda):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    g = Golden("pp2k", cuda)
    G = cuda.Graph(g.x)
    S = g.x.span
    off = _dev(torch, g.x.offsets.astype(np.uint64), np.int64)
    key = _dev(torch, g.x.keys.astype(np.uint32), np.int32)
    w = _dev(torch, g.x.weights.astype(np.float32), np.float32)
    ex = _dev(torch, g.x.exists.astype(np.uint8), np.uint8)
    out = torch.full((1,), -7.0, dtype=torch.float64, device="cuda:0")
    ids = np.arange(S, dtype=np.uint32)
    ids[~g.x.exists.astype(bool)] = 0
    memberships = [g["static_m"].astype(np.uint32), ids]  # the reference's result, then singletons
    for memb in memberships:
        m = _dev(torch, memb, np.int32)
        torch.cuda.synchronize()
        cuda.modularity_noalloc(S, off.data_ptr(), key.data_ptr(), w.data_ptr(), ex.data_ptr(), m.data_ptr(),
                                out.data_ptr())
        torch.cuda.synchronize()
        expect = G.modularity(memb)
        assert abs(out.item() - expect) <= TOL, (out.item(), expect)


def test_noalloc_rejects_spans_above_its_limit(cuda):
    with pytest.raises(cuda.LvgError) as e:
        cuda.modularity_noalloc(cuda.NOALLOC_MAX_SPAN + 1, 1, 1, 1, None, 1, 1)
    assert e.value.code == cuda.LVG_EINVAL


def test_noalloc_out_of_range_id_gives_nan(cuda):
    """A membership id >= span is not a valid community: the result is NaN,
    not a read past the caller's buffers. A call after it is correct again
    (the shared scratch is cleared by every call)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    g = Golden("pp2k", cuda)
    S = g.x.span
    off = _dev(torch, g.x.offsets.astype(np.uint64), np.int64)
    key = _dev(torch, g.x.keys.astype(np.uint32), np.int32)
    w = _dev(torch, g.x.weights.astype(np.float32), np.float32)
    out = torch.full((1,), -7.0, dtype=torch.float64, device="cuda:0")
    memb = g["static_m"].astype(np.uint32).copy()
    bad = memb.copy()
    bad[int(np.flatnonzero(g.x.exists)[0])] = S  # one id past the span
    m = _dev(torch, bad, np.int32)
    torch.cuda.synchronize()
    cuda.modularity_noalloc(S, off.data_ptr(), key.data_ptr(), w.data_ptr(), None, m.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    assert np.isnan(out.item())
    m = _dev(torch, memb, np.int32)
    cuda.modularity_noalloc(S, off.data_ptr(), key.data_ptr(), w.data_ptr(), None, m.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    assert abs(out.item() - cuda.Graph(g.x).modularity(memb)) <= TOL


def test_noalloc_rejects_null_edge_arrays(cuda):
    # checked on the host before anything is launched
    for keys, weights in ((0, 1), (1, 0)):
        with pytest.raises(cuda.LvgError) as e:
            cuda.modularity_noalloc(16, 1, keys, weights, None, 1, 1)
        assert e.value.code == cuda.LVG_EINVAL
