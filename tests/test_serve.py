"""Serving engine (pg_engine_*): continuous batching of single points.

Each request is one ClusterAnion::EnergyFromConfiguration-style single point
(src/ClusterAnion.cpp:192-290): water cluster -> V(r) -> Davidson.  The tests
check that
  - a solve's result is the same alone and in a mix of concurrent solves on
    the same and on different grids (bit for bit: merged tensor-core launches
    compute every column as a launch of its own would), also with the
    kinetic preconditioner, whose launches from several solves overlap;
  - the engine's solve equals the single-call path pg_cluster_solve;
  - admission keeps the admitted footprint within the memory budget and
    rejects a request that can never fit;
  - warm start from the cached eigenvectors of the same key needs fewer H*x
    products than a cold start and lands on the same states;
  - bad requests fail at submit, and a solve that runs out of iterations
    reports PG_NOT_CONVERGED in its result.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRID = (40, 40, 40)
L40 = 0.615 * 41


@pytest.fixture(scope="module")
def torch():
    import torch
    assert torch.cuda.is_available()
    return torch


@pytest.fixture(scope="module")
def mix(clusters):
    """Five seeded clusters: four on a 40^3 grid, one on 48^3."""
    out = []
    for i, nw in enumerate((6, 8, 10, 12, 8)):
        w = clusters.water_cluster(nw, 5.0 + 0.2 * nw, seed=100 + i)
        grid = GRID if i < 4 else (48, 48, 48)
        L = L40 if i < 4 else 0.615 * 49
        out.append((w, grid, L, 1 + i % 3))
    return out


def _run(pg, reqs, **cfg):
    with pg.Engine(**cfg) as eng:
        ids = [eng.submit(r) for r in reqs]
        res = [eng.wait(i, timeout=300.0) for i in ids]
        stats = eng.stats()
    return res, stats


def _requests(pg, mix, precision):
    return [pg.Engine.request(grid, L, w, nroots=nr, maxsub=40, ptol=6, precision=precision, want_vectors=True)
            for (w, grid, L, nr) in mix]


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_alone_equals_in_the_mix(pg, torch, mix, precision):
    alone = []
    for r in _requests(pg, mix, precision):
        res, _ = _run(pg, [r], slots=1, warm_start=False)
        alone.append(res[0])
    together, stats = _run(pg, _requests(pg, mix, precision), slots=8, warm_start=False, batch_window_us=2000)
    assert all(a["status"] == 0 for a in alone), [a["error"] for a in alone]
    assert stats["completed"] == len(mix) and stats["failed"] == 0, [b["error"] for b in together]
    assert stats["peak_in_flight"] > 1
    if precision == 1:
        # products of the four 40^3 solves went through merged launches
        assert stats["batched_products"] > stats["batches"]
    for a, b in zip(alone, together):
        assert a["status"] == 0 and b["status"] == 0, (a["error"], b["error"])
        assert a["evals"] == b["evals"]
        assert np.array_equal(a["vectors"], b["vectors"])
        assert a["stats"]["n_matvec"] == b["stats"]["n_matvec"]


def test_alone_equals_in_the_mix_kinetic_preconditioner(pg, torch, mix):
    # the mixed form with corrflag 3: every solve runs the FP16-split H*X
    # (merged across solves) and the FP16 kinetic preconditioner, whose
    # launches from the eight slots overlap on the device; each solve must
    # still give the bits it gives alone
    def reqs():
        return [pg.Engine.request(grid, L, w, nroots=nr, maxsub=40, maxiter=400, ptol=6, corrflag=3, precision=1,
                                  want_vectors=True) for (w, grid, L, nr) in mix]
    alone = [_run(pg, [r], slots=1, warm_start=False)[0][0] for r in reqs()]
    together, stats = _run(pg, reqs(), slots=8, warm_start=False, batch_window_us=2000)
    assert stats["peak_in_flight"] > 1
    assert sum(a["status"] == 0 for a in alone) >= 3, [a["error"] for a in alone]
    for a, b in zip(alone, together):
        assert a["status"] == b["status"], (a["error"], b["error"])
        if a["status"] == 0:
            assert a["evals"] == b["evals"]
            assert np.array_equal(a["vectors"], b["vectors"])
            assert a["stats"]["n_matvec"] == b["stats"]["n_matvec"]


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_engine_equals_single_call(pg, torch, mix, precision):
    w, grid, L, nr = mix[1]
    res, _ = _run(pg, [pg.Engine.request(grid, L, w, nroots=nr, maxsub=40, ptol=6, precision=precision,
                                         want_vectors=True)], slots=2)
    ev, vec, _ = pg.cluster_solve(grid, [L] * 3, w, nroots=nr, maxsub=40, ptol=6, precision=precision)
    assert res[0]["evals"] == list(ev)
    assert np.array_equal(res[0]["vectors"], vec)


def test_mixed_agrees_with_fp64(pg, torch, mix):
    r64, _ = _run(pg, _requests(pg, mix, 0), slots=8, warm_start=False)
    rmx, _ = _run(pg, _requests(pg, mix, 1), slots=8, warm_start=False)
    for a, b in zip(r64, rmx):
        assert max(abs(x - y) for x, y in zip(a["evals"], b["evals"])) <= 1e-6


def test_admission_by_footprint(pg, torch, mix):
    reqs = _requests(pg, mix[:4], 1)
    fp = max(pg.Engine.footprint(r) for r in reqs)
    res, stats = _run(pg, reqs, slots=4, memory_budget=1.5 * fp, warm_start=False)
    assert all(r["status"] == 0 for r in res)
    assert stats["peak_in_flight"] == 1 and stats["peak_bytes"] <= 1.5 * fp
    res, stats = _run(pg, _requests(pg, mix[:4], 1), slots=4, memory_budget=2.5 * fp, warm_start=False)
    assert stats["peak_in_flight"] <= 2 and stats["peak_bytes"] <= 2.5 * fp
    with pg.Engine(slots=2, memory_budget=0.5 * fp) as eng:
        with pytest.raises(pg.PiscesError) as e:
            eng.submit(reqs[0])
        assert e.value.status == pg.PG_OOM


def test_warm_start_same_key(pg, torch, clusters):
    rng = np.random.Generator(np.random.PCG64(7))
    base = clusters.water_cluster(10, 7.0, seed=41)
    snaps = [clusters.jitter(base, rng) for _ in range(3)]
    kw = dict(nroots=2, maxsub=40, ptol=6, precision=1)
    cold, _ = _run(pg, [pg.Engine.request(GRID, L40, s, key=-1, **kw) for s in snaps], slots=1)
    with pg.Engine(slots=1) as eng:
        warm = [eng.wait(eng.submit(pg.Engine.request(GRID, L40, s, key=5, **kw)), timeout=300.0) for s in snaps]
        stats = eng.stats()
    assert [r["warm_started"] for r in warm] == [False, True, True]
    assert stats["warm_starts"] == 2
    for c, w in zip(cold[1:], warm[1:]):
        assert w["stats"]["n_matvec"] < c["stats"]["n_matvec"]
        assert max(abs(x - y) for x, y in zip(c["evals"], w["evals"])) <= 1e-6


def test_bad_requests(pg, torch, mix):
    w, grid, L, _ = mix[0]
    bad = np.array(w, dtype=np.float64)
    bad[0, 1] = np.nan
    with pg.Engine(slots=2) as eng:
        with pytest.raises(pg.PiscesError) as e:
            eng.submit(pg.Engine.request(grid, L, bad, nroots=1))
        assert e.value.status == pg.PG_BAD_ARG
        with pytest.raises(pg.PiscesError) as e:
            eng.submit(pg.Engine.request((260, 260, 260), 160.0, w, nroots=1, precision=1))
        assert e.value.status == pg.PG_UNSUPPORTED
        rid = eng.submit(pg.Engine.request(grid, L, w, nroots=2, maxiter=1, ptol=10))
        r = eng.wait(rid, timeout=300.0)
        assert r["status"] == pg.PG_NOT_CONVERGED and "converged" in r["error"]
        assert r["stats"]["nconv"] < 2
        # the engine keeps serving after a failed request
        ok = eng.wait(eng.submit(pg.Engine.request(grid, L, w, nroots=1, maxsub=40, ptol=6)), timeout=300.0)
        assert ok["status"] == 0


def test_poll_and_wait_hand_over_once(pg, torch, mix):
    with pg.Engine(slots=4) as eng:
        ids = [eng.submit(r) for r in _requests(pg, mix[:3], 1)]
        first = eng.wait(ids[0], timeout=300.0)
        got = {first["id"]}
        while len(got) < 3:
            time.sleep(0.01)
            for r in eng.poll():
                assert r["id"] not in got
                got.add(r["id"])
        with pytest.raises(pg.PiscesError):
            eng.wait(ids[1], timeout=1.0)
    assert got == set(ids)


def test_warm_start_fills_missing_states(pg, torch, clusters):
    """A cached entry with fewer states than asked for seeds the leading
    columns; the request's own start vectors fill the rest."""
    w = clusters.water_cluster(10, 7.0, seed=43)
    kw = dict(maxsub=40, ptol=6, precision=1)
    cold, _ = _run(pg, [pg.Engine.request(GRID, L40, w, nroots=3, key=-1, **kw)], slots=1)
    with pg.Engine(slots=1) as eng:
        one = eng.wait(eng.submit(pg.Engine.request(GRID, L40, w, nroots=1, key=9, **kw)), timeout=300.0)
        three = eng.wait(eng.submit(pg.Engine.request(GRID, L40, w, nroots=3, key=9, **kw)), timeout=300.0)
        again = eng.wait(eng.submit(pg.Engine.request(GRID, L40, w, nroots=1, key=9, **kw)), timeout=300.0)
    assert not one["warm_started"] and three["warm_started"] and again["warm_started"]
    assert three["status"] == 0
    assert max(abs(x - y) for x, y in zip(cold[0]["evals"], three["evals"])) <= 1e-6
    assert abs(again["evals"][0] - cold[0]["evals"][0]) <= 1e-6
    # the same geometry again: the cached vectors are already converged
    assert again["stats"]["n_matvec"] < one["stats"]["n_matvec"]
