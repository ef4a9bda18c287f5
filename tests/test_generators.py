"""Graphs and batches generated in HBM against the host generators.

The device generators (lvg_graph_create_planted_partition / _rmat,
lvg_device_batch_generate) draw from the same counter-based streams as the
host ones (lvgg_planted_partition / lvgg_rmat / lvgg_reference_batch), so the
results must be equal entry for entry. The batch generator mirrors the
reference's generateEdgeDeletions / generateEdgeInsertions
(inc/batch.hxx:105-143); a device batch then goes through the device tidy and
apply and must equal the oracle's tidyBatchUpdateU + applyBatchUpdateOmpU.
"""
import numpy as np
import pytest


def _same_graph(h, x):
    assert np.array_equal(h.offsets, x.offsets)
    assert np.array_equal(h.keys, x.keys)
    assert np.array_equal(h.weights, x.weights)
    assert np.array_equal(h.exists, x.exists)


# ------------------------------------------------------------------- CPU

def test_reference_batch_draws_as_the_reference_does(lvg):
    x = lvg.planted_partition(3000, 100, 10, 0.8, 5)
    b = lvg.reference_batch(x, 400, 1600, begin=1, range_=3000, weight=2.0, seed=11)
    # both directions, pairwise
    assert b.num_deletions % 2 == 0 and b.num_insertions == 3200
    assert np.array_equal(b.del_src[0::2], b.del_dst[1::2]) and np.array_equal(b.del_dst[0::2], b.del_src[1::2])
    assert np.array_equal(b.ins_src[0::2], b.ins_dst[1::2]) and np.array_equal(b.ins_dst[0::2], b.ins_src[1::2])
    # insertions uniform in the range with the given weight; deletions are edges of x with their weights
    assert b.ins_src.min() >= 1 and b.ins_src.max() <= 3000 and np.all(b.ins_w == 2.0)
    off = x.offsets.astype(np.int64)
    for u, v, w in zip(b.del_src.astype(np.int64), b.del_dst, b.del_w):
        row = x.keys[off[u]:off[u + 1]]
        j = int(np.searchsorted(row, v))
        assert j < len(row) and row[j] == v and x.weights[off[u] + j] == w
    # every source has edges here, so no draw fails
    assert b.num_deletions == 800
    # deterministic in the seed
    c = lvg.reference_batch(x, 400, 1600, begin=1, range_=3000, weight=2.0, seed=11)
    assert np.array_equal(b.ins_dst, c.ins_dst) and np.array_equal(b.del_dst, c.del_dst)


def test_reference_batch_rejects_a_range_outside_the_span(lvg):
    x = lvg.planted_partition(100, 10, 4, 0.8, 5)
    with pytest.raises(lvg.LvgError):
        lvg.reference_batch(x, 1, 1, begin=50, range_=60)


# ------------------------------------------------------------------- GPU

@pytest.mark.gpu
@pytest.mark.parametrize("n,block,deg,p,seed", [(2048, 128, 16, 0.8, 11), (5000, 37, 9.5, 0.6, 3)])
def test_device_planted_partition_equals_host(cuda, n, block, deg, p, seed):
    G = cuda.Graph.planted_partition(n, block, deg, p, seed)
    x = cuda.planted_partition(n, block, deg, p, seed)
    _same_graph(G.download(), x)
    assert G.order == n and G.size == x.num_edges


@pytest.mark.gpu
@pytest.mark.parametrize("scale,ef,permute", [(12, 16, True), (14, 8, False)])
def test_device_rmat_equals_host(cuda, scale, ef, permute):
    G = cuda.Graph.rmat(scale, ef, permute=permute, seed=5)
    x = cuda.rmat(scale, ef, seed=5, permute=permute)
    _same_graph(G.download(), x)
    assert G.edge_weight() == float(x.num_edges)


@pytest.mark.gpu
def test_device_batch_generator_equals_host_and_applies_like_the_oracle(cuda, orc):
    x = cuda.rmat(12, 8, seed=9)
    G = cuda.Graph(x)
    db = cuda.DeviceBatch.generate(G, 3000, 12000, begin=1, range_=x.span - 1, weight=1.0, seed=21)
    hb = cuda.reference_batch(x, 3000, 12000, begin=1, range_=x.span - 1, weight=1.0, seed=21)
    d = db.download()
    for k in ("del_src", "del_dst", "del_w", "ins_src", "ins_dst", "ins_w"):
        assert np.array_equal(getattr(d, k), getattr(hb, k)), k
    G.apply_batch(db)
    (yo, yk, yw, yex), tidy = orc.apply_batch(x, hb)
    h = G.download()
    assert np.array_equal(h.offsets, yo) and np.array_equal(h.keys, yk) and np.array_equal(h.weights, yw)
    assert np.array_equal(h.exists, yex)
    t = db.download()  # the device batch is now the tidied batch
    for a, k in zip(tidy, ("del_src", "del_dst", "del_w", "ins_src", "ins_dst", "ins_w")):
        assert np.array_equal(a, getattr(t, k)), k
