"""GPU: the serving loop -- every request's result is the same alone and in a mix of
resident / uploaded, weighted / unweighted, vertex- / edge-centric requests that queue, fold
into shared passes and overlap on several streams; admission by the memory budget."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def pool(jx):
    graphs = []
    for i, sc in enumerate([10, 11, 12, 13, 14, 12]):
        rp, col = jx.graphgen.rmat(sc, 16, seed=600 + i)
        graphs.append((rp, col, jx.graphgen.uniform_weights(len(rp) - 1, seed=700 + i)))
    uploads = []
    rng = np.random.default_rng(8)
    for i in range(10):
        n = int(rng.integers(100, 20000))
        if i % 2:
            rp, col = jx.graphgen.er_gnm(n, n * int(rng.integers(2, 30)), seed=800 + i)
        else:
            rp, col = jx.graphgen.rmat(int(np.log2(n)) + 1, int(rng.integers(4, 20)), seed=800 + i)
        uploads.append((rp, col, jx.graphgen.uniform_weights(len(rp) - 1, seed=900 + i)))
    return graphs, uploads


def oracle_of(O, g, weighted, ec):
    rp, col, w = g
    return O.jaccard(rp, col, w if weighted else None, edge_centric=ec)


def alone(jx, g, weighted, ec):
    import torch
    rp, col, w = g
    view = jx.GraphCSRView.from_numpy(rp, col)
    return jx.jaccard(view, torch.from_numpy(w).cuda() if weighted else None, edge_centric=ec).cpu().numpy()


@pytest.mark.parametrize("schedule", [None, {"persistent": 1}], ids=["per-bin", "persistent"])
def test_mix_equals_alone(jx, O, pool, schedule):
    graphs, uploads = pool
    srv = jx.Server(memory_budget=4 << 30, slots=3, fold_edges=200_000, fold_max_edges=2_000_000,
                    schedule=schedule)
    ids = [srv.add_graph(*g) for g in graphs]
    rng = np.random.default_rng(9)
    reqs = []
    for i in range(80):
        weighted = bool(rng.integers(0, 4))  # mostly weighted
        ec = (not weighted) and bool(rng.integers(0, 2))
        if rng.random() < 0.6:
            k = int(rng.integers(0, len(graphs)))
            reqs.append((ids[k], graphs[k], weighted, ec))
        else:
            k = int(rng.integers(0, len(uploads)))
            reqs.append((uploads[k], uploads[k], weighted, ec))
    outs = []
    tickets = []
    for target, g, weighted, ec in reqs:  # all at once: they queue, fold and overlap
        out = np.empty(len(g[1]), np.float32)
        outs.append(out)
        tickets.append(srv.submit(target, out, weighted=weighted, edge_centric=ec))
    lat = [srv.wait(t) for t in tickets]
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["passes"] < len(reqs) and st["folded_requests"] > 0
    assert st["p99_ms"] >= st["p50_ms"] > 0 and max(lat) <= st["max_ms"] + 1e-6
    # every request against the oracle on its graph, and against the graph scored alone
    cache = {}
    for (target, g, weighted, ec), out in zip(reqs, outs):
        key = (id(g), weighted, ec)
        if key not in cache:
            cache[key] = (oracle_of(O, g, weighted, ec), alone(jx, g, weighted, ec))
        want, one = cache[key]
        assert np.array_equal(bits(out), bits(want)), f"request differs from the oracle (weighted={weighted}, ec={ec})"
        assert np.array_equal(bits(one), bits(want))
    # the same requests one at a time through the server
    for (target, g, weighted, ec), out in list(zip(reqs, outs))[:12]:
        one = np.empty_like(out)
        srv.wait(srv.submit(target, one, weighted=weighted, edge_centric=ec))
        assert np.array_equal(bits(one), bits(out))
    srv.close()


def test_admission_budget(jx, pool):
    graphs, _ = pool
    rp, col, w = graphs[4]  # RMAT scale 14: about 3.6 MB of device memory unweighted
    small = jx.graphgen.er_gnm(1000, 4000, seed=11)  # about 0.1 MB
    srv = jx.Server(memory_budget=2 << 20, slots=2)
    big_out = np.empty(len(col), np.float32)
    t_big = srv.submit((rp, col), big_out)
    out = np.empty(len(small[1]), np.float32)
    t_small = srv.submit(small, out)
    with pytest.raises(jx.JxError) as e:
        srv.wait(t_big)
    assert e.value.status == 6  # JX_ERR_TOO_LARGE: above the whole budget
    srv.wait(t_small)
    assert np.array_equal(bits(out), bits(alone(jx, (small[0], small[1], None), False, False)))
    # a weighted request on a graph kept without weights is refused at submit
    gid = srv.add_graph(small[0], small[1])
    with pytest.raises(jx.JxError):
        srv.submit(gid, np.empty(len(small[1]), np.float32), weighted=True)
    srv.close()


def test_injected_alloc_failure_fails_one_pass_only(jx, O, pool):
    """An allocation failure inside one pass (injected on the host) fails that pass's request
    with JX_ERR_NOMEM; every other request completes bit for bit, and the failed one succeeds
    when submitted again."""
    graphs, _ = pool
    srv = jx.Server(memory_budget=2 << 30, slots=2, fold_edges=0)  # no folding: a pass per request
    ids = [srv.add_graph(*g) for g in graphs[:4]]
    srv.pause()
    outs = [np.empty(len(g[1]), np.float32) for g in graphs[:4]]
    tickets = [srv.submit(gid, out, weighted=True) for gid, out in zip(ids, outs)]
    srv.inject_alloc_failures(1)
    srv.pause(False)
    failed = []
    for k, t in enumerate(tickets):
        try:
            srv.wait(t)
        except jx.JxError as e:
            assert e.status == 3  # JX_ERR_NOMEM
            failed.append(k)
    assert len(failed) == 1
    for k, (rp, col, w) in enumerate(graphs[:4]):
        if k not in failed:
            assert np.array_equal(bits(outs[k]), bits(O.jaccard(rp, col, w)))
    k = failed[0]
    again = np.empty_like(outs[k])
    srv.wait(srv.submit(ids[k], again, weighted=True))
    assert np.array_equal(bits(again), bits(O.jaccard(*graphs[k])))
    st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 4
    srv.close()


def test_cancel_queued_request(jx, O, pool):
    """A request cancelled while it waits in the queue never runs: its wait reports
    JX_ERR_CANCELLED and its host buffer is untouched; the requests around it complete bit for
    bit.  Requests that have finished can no longer be cancelled."""
    graphs, uploads = pool
    srv = jx.Server(memory_budget=2 << 30, slots=1)
    srv.pause()
    reqs = [graphs[0], uploads[1], graphs[2]]
    outs = [np.full(len(g[1]), np.nan, np.float32) for g in reqs]
    tickets = [srv.submit(g, out, weighted=True) for g, out in zip(reqs, outs)]
    assert srv.cancel(tickets[1]) is True
    srv.pause(False)
    for k in (0, 2):
        srv.wait(tickets[k])
        assert np.array_equal(bits(outs[k]), bits(O.jaccard(*reqs[k])))
    with pytest.raises(jx.JxError) as e:
        srv.wait(tickets[1])
    assert e.value.status == 7
    assert np.all(np.isnan(outs[1]))
    t = srv.submit(uploads[0], np.empty(len(uploads[0][1]), np.float32), weighted=True)
    srv.drain()
    assert srv.cancel(t) is False  # finished: nothing to cancel
    srv.wait(t)
    with pytest.raises(jx.JxError):
        srv.cancel(t)  # unknown after its wait
    st = srv.stats()
    assert st["cancelled"] == 1 and st["failed"] == 0 and st["completed"] == 3
    srv.close()
