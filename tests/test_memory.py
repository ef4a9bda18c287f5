"""Device-memory accounting per handle (lvg_graph_device_bytes and friends)
and lvg_graph_trim: what the serving loop's admission control measures."""
import numpy as np
import pytest


@pytest.mark.gpu
def test_device_bytes_follow_allocations_and_trim(cuda):
    x = cuda.planted_partition(8192, 128, 16, 0.8, 7)
    G = cuda.Graph(x)
    b0 = G.device_bytes()
    assert b0 >= 8 * x.num_edges + 16 * x.span  # rows (id + weight) and per-vertex arrays
    o = cuda.LouvainOptions(deterministic=True)
    r1 = cuda.louvain_static(G, o)
    b1 = G.device_bytes()
    assert b1 > b0  # the workspace
    G.trim(1)
    b2 = G.device_bytes()
    assert b2 <= b1
    G.trim(2)
    b3 = G.device_bytes()
    assert b3 < b2
    r2 = cuda.louvain_static(G, o)  # works again after the trim, same result
    assert np.array_equal(r1.membership, r2.membership)
    st = cuda.State(G)
    assert cuda.load_library().lvg_state_device_bytes(st.h) >= x.span * 12
    db = cuda.DeviceBatch(G, cuda.random_batch(x, 500, 0.8, seed=3))
    assert cuda.load_library().lvg_device_batch_device_bytes(db.h) > 0
    G.close()  # the batch and the state outlive the graph
    db.close()
    st.close()
