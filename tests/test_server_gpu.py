"""Build server (nxb_server_*): every request's BVH8 equals a plain build of
that mesh alone, whether the server built it alone or batched with others;
admission keeps the server inside its memory budget."""
import numpy as np
import pytest

import nexusbvh_gb300 as nxb
from nexusbvh_gb300 import scenes
from tests import stages as S

pytestmark = pytest.mark.gpu


def plain_bvh8(prims, key_bits, radius=8):
    out = S.build_async(prims, key_bits, radius=radius)
    b8 = S.host(out.nodes.reshape(-1)).view(nxb.BVH8_NODE_DTYPE)
    prim = S.host(out.prim_idx).view(np.uint32)
    return b8, prim, out.bounds


def check_same(orc, res, prims, key_bits):
    assert res.status == 0
    n = prims.shape[0]
    b8, prim = nxb.Server.bvh8_host(res)
    b8p, primp, bounds = plain_bvh8(prims, key_bits)
    assert res.bvh8.node_count == b8p.shape[0] and res.bvh8.prim_count == n
    assert orc.compare_bvh8(b8, prim, b8p, primp, n) == 0
    assert tuple(res.bvh8.bounds.bmin) == bounds[0] and tuple(res.bvh8.bounds.bmax) == bounds[1]


def mixed_requests(seed=0):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(24):
        n = int(rng.integers(1, 3000)) if i % 4 else int(rng.integers(20_000, 90_000))
        kind = i % 3
        if kind == 0:
            p = scenes.uniform_soup(n, seed=100 + i)
        elif kind == 1:
            p = scenes.clustered(n, seed=200 + i, components=8)
        else:
            p = scenes.batch_meshes([n], seed=300 + i)
        key_bits = 63 if i % 5 == 0 else 30
        reqs.append((p, key_bits))
    reqs.append((scenes.to_boxes(scenes.uniform_soup(1500, seed=7)), 30))
    reqs.append((scenes.to_boxes(scenes.uniform_soup(700, seed=8)), 30))
    return reqs


def test_server_results_match_plain_builds(gpu, orc):
    srv = nxb.Server(streams=1)
    # a large request first, so that the small ones queue behind it and get batched
    big = scenes.clustered(2_000_000, seed=3)
    t_big = srv.submit(big, nxb.BuildConfig(prioritize_speed=True))
    reqs = mixed_requests()
    tickets = []
    for k, (p, kb) in enumerate(reqs):
        src = p if k % 2 else S.dev(p)  # host and device inputs
        tickets.append(srv.submit(src, nxb.BuildConfig(prioritize_speed=kb == 30)))
    r_big = srv.wait(t_big)
    check_same(orc, r_big, big, 30)
    srv.release(t_big)
    batched = 0
    for t, (p, kb) in zip(tickets, reqs):
        r = srv.wait(t)
        check_same(orc, r, p, kb)
        batched += r.batched_with > 1
        srv.release(t)
    st = srv.stats()
    assert st.completed == len(reqs) + 1 and st.submitted == len(reqs) + 1
    assert st.batched_builds >= 1 and batched >= 2
    assert st.bytes_in_use == 0
    srv.close()


def test_server_same_tree_alone_and_mixed(gpu, orc):
    x = scenes.batch_meshes([2500], seed=42)
    srv = nxb.Server()
    t = srv.submit(x, nxb.BuildConfig(prioritize_speed=True))
    alone = srv.wait(t)
    assert alone.batched_with == 1
    a8, ap = nxb.Server.bvh8_host(alone)
    srv.release(t)
    srv.close()
    srv = nxb.Server(streams=1)
    t_big = srv.submit(scenes.clustered(1_000_000, seed=4), nxb.BuildConfig(prioritize_speed=True))
    others = [srv.submit(scenes.uniform_soup(300 + 50 * i, seed=i), nxb.BuildConfig(prioritize_speed=True))
              for i in range(10)]
    t = srv.submit(x, nxb.BuildConfig(prioritize_speed=True))
    more = [srv.submit(scenes.uniform_soup(800, seed=50 + i), nxb.BuildConfig(prioritize_speed=True))
            for i in range(5)]
    mixed = srv.wait(t)
    assert mixed.batched_with > 1
    m8, mp = nxb.Server.bvh8_host(mixed)
    assert orc.compare_bvh8(a8, ap, m8, mp, 2500) == 0
    assert orc.digest_bvh8(a8, ap, 2500) == orc.digest_bvh8(m8, mp, 2500)
    for k in [t_big, t] + others + more:
        srv.wait(k)
        srv.release(k)
    srv.close()


def test_server_mixed_batch_matches_oracle(gpu, orc):
    """Requests that the server builds together in one batched launch each
    equal the oracle's tree for that mesh alone: the oracle's H-PLOC and
    BVH8 collapse (oracle/nxb_oracle.cpp) over the mesh's own GPU Morton
    order, which run_chain checks stage by stage."""
    from tests.test_gpu_parity import run_chain
    srv = nxb.Server(streams=1)
    t_big = srv.submit(scenes.clustered(1_500_000, seed=6), nxb.BuildConfig(prioritize_speed=True))
    meshes = [scenes.uniform_soup(700 + 311 * i, seed=60 + i) if i % 3 == 0 else
              scenes.clustered(500 + 173 * i, seed=70 + i, components=6) if i % 3 == 1 else
              scenes.batch_meshes([900 + 97 * i], seed=80 + i) for i in range(9)]
    tickets = [srv.submit(m if i % 2 else S.dev(m), nxb.BuildConfig(prioritize_speed=True))
               for i, m in enumerate(meshes)]
    srv.wait(t_big)
    srv.release(t_big)
    checked = 0
    for t, m in zip(tickets, meshes):
        r = srv.wait(t)
        assert r.status == 0
        n = m.shape[0]
        b8, prim = nxb.Server.bvh8_host(r)
        chain = run_chain(m, 30, orc)
        b8_o, prim_o, err = orc.bvh8(chain["b2"], n, 2 * n - 2)
        assert err == 0
        assert orc.compare_bvh8(b8, prim, b8_o, prim_o, n) == 0
        checked += r.batched_with > 1
        srv.release(t)
    assert checked >= 2, "the small requests were expected to be built together"
    srv.close()


def intervals_overlap(a, b):
    return max(a.device_start_ms, b.device_start_ms) < min(a.device_end_ms, b.device_end_ms)


def test_server_requests_overlap_on_the_device(gpu, orc):
    """Continuous batching runs requests at the same time: with four stream
    slots, requests submitted together have GPU work at the same time (their
    device intervals, from events on their streams, intersect), and each
    result is still the mesh's plain build.  Requests built together share
    one interval."""
    srv = nxb.Server(streams=4, batch_max_prims=1)  # every request its own build
    meshes = [scenes.clustered(400_000 + 10_000 * i, seed=90 + i) for i in range(8)]
    tickets = [srv.submit(S.dev(m), nxb.BuildConfig()) for m in meshes]
    res = []
    for t, m in zip(tickets, meshes):
        r = srv.wait(t)
        assert 0.0 <= r.device_start_ms < r.device_end_ms
        check_same(orc, r, m, 63)
        res.append(r)
        srv.release(t)
    srv.close()
    pairs = [(i, j) for i in range(len(res)) for j in range(i + 1, len(res)) if intervals_overlap(res[i], res[j])]
    assert pairs, "no two requests had work on the GPU at the same time"

    srv = nxb.Server(streams=1)
    t_big = srv.submit(scenes.clustered(1_000_000, seed=5), nxb.BuildConfig(prioritize_speed=True))
    small = [srv.submit(scenes.uniform_soup(500 + 100 * i, seed=i), nxb.BuildConfig(prioritize_speed=True))
             for i in range(6)]
    srv.wait(t_big)
    srv.release(t_big)
    rs = []
    for t in small:
        rs.append(srv.wait(t))
    together = [r for r in rs if r.batched_with > 1]
    assert len(together) >= 2
    assert all(r.device_start_ms == together[0].device_start_ms for r in together[:2])
    for t in small:
        srv.release(t)
    srv.close()


def test_server_admission_and_budget(gpu, orc):
    budget = 96 << 20
    srv = nxb.Server(budget_bytes=budget, streams=4, batch_max_prims=1)  # no batching: plain builds only
    with pytest.raises(nxb.NxbError) as ei:
        srv.submit(scenes.uniform_soup(2_000_000, seed=1), nxb.BuildConfig(prioritize_speed=True))
    assert ei.value.status == 8
    meshes = [scenes.uniform_soup(200_000, seed=10 + i) for i in range(8)]
    tickets = [srv.submit(m, nxb.BuildConfig(prioritize_speed=True)) for m in meshes]
    for t, m in zip(tickets, meshes):
        r = srv.wait(t)
        check_same(orc, r, m, 30)
        srv.release(t)
    st = srv.stats()
    assert st.rejected == 1 and st.completed == 8
    assert 0 < st.peak_bytes_in_use <= budget
    assert st.bytes_in_use == 0
    srv.close()


def test_server_poll_and_errors(gpu):
    srv = nxb.Server()
    t = srv.submit(scenes.uniform_soup(5000, seed=2), nxb.BuildConfig(prioritize_speed=True))
    r = None
    for _ in range(100000):
        r = srv.poll(t)
        if r is not None:
            break
    if r is None:
        r = srv.wait(t)
    assert r.status == 0
    srv.release(t)
    with pytest.raises(nxb.NxbError):
        srv.release(t)  # already released
    with pytest.raises(nxb.NxbError):
        srv.submit(scenes.uniform_soup(10), nxb.BuildConfig(prioritize_speed=True, search_radius=5))
    srv.close()
