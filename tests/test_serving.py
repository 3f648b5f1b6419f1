"""The continuous-batching server (include/cy_serve.h): every request's
result is the same whether it is rendered alone or in a mix that arrives
while other frames are on the GPU; admission respects the memory budget."""
import numpy as np
import pytest

from canvas_ity_gb300 import native, scenes, serving
import golden_util as G
import oracle

pytestmark = pytest.mark.gpu


def _requests(n, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        w, h = int(rng.integers(32, 320)), int(rng.integers(32, 320))
        out.append(scenes.mixed_canvas(scenes.BASE_SEED + 31 * i + seed, w, h, int(rng.integers(1, 40)),
                                       clip=bool(i % 5 == 0)))
    return out


def test_each_result_same_alone_and_in_the_mix():
    reqs = _requests(40)
    alone = [native.render_batch([t], 0)[0] for t in reqs]
    with serving.Server(workers=3, max_batch=16) as srv:
        res = serving.run_poisson(srv, reqs, rate=4000.0, seed=1, keep_results=True)
        stats = srv.stats()
    assert res["failed"] == 0
    assert stats["frames"] > 1            # the mix really was split over several frames
    for tb, a, r in zip(reqs, alone, res["results"]):
        assert r.status == 0
        assert r.images == a              # bit-identical to rendering it alone
    # and within the parity tolerance of the oracle
    for tb, r in list(zip(reqs, res["results"]))[::8]:
        for g, w in zip(G.split_images(tb, r.images), G.split_images(tb, oracle.replay(tb)[0])):
            G.assert_within_contract(g, w, "served request")


def test_admission_budget_limits_what_runs_at_once():
    reqs = _requests(12, seed=3)
    budget = 64 << 20     # 64 MiB: only a few small requests fit at once
    with serving.Server(budget_bytes=budget, workers=4, max_batch=64) as srv:
        ids = [srv.submit(t) for t in reqs]
        got = {}
        while len(got) < len(ids):
            r = srv.poll(2000)
            assert r is not None
            got[r.id] = r
        stats = srv.stats()
    assert all(r.status == 0 for r in got.values())
    assert stats["max_bytes_admitted"] <= budget
    assert stats["requests"] == len(reqs)
    for rid, tb in zip(ids, reqs):
        assert got[rid].images == native.render_batch([tb], 0)[0]
