"""The serving loop on the GPU: concurrent requests of two models (blackbody
and Num4D) with continuous batching; each request's result is the same alone
and in the mix (to round-off: the parallels of a mesh may be chunked
differently in a bigger launch)."""
import numpy as np
import pytest

from batch_cases import small_blackbody, small_num4d

pytestmark = pytest.mark.gpu


def test_same_alone_and_in_the_mix():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xpsi_gb300.serving import Server
    mn, pn = small_num4d(V=6)
    mb, pb = small_blackbody(V=5)
    srv = Server({"num4d": mn, "bb": mb}, slots=3, hbm_budget=8 << 30)
    try:
        alone = [srv.submit("num4d", pn[i:i + 1]).result(timeout=120) for i in range(2)]
        alone_bb = srv.submit("bb", pb[0:1]).result(timeout=120)
        futs = [srv.submit("num4d", pn[i:i + 1]) for i in range(6)]
        futs += [srv.submit("bb", pb[i:i + 1]) for i in range(5)]
        futs.append(srv.submit("num4d", pn))
        futs.append(srv.submit("num4d", pn[:3]))
        futs.append(srv.submit("num4d", pn[3:5]))
        res = [f.result(timeout=300) for f in futs]
    finally:
        srv.close()
    for i in range(2):
        ll_a, st_a = alone[i]
        ll_m, st_m = res[i]
        assert st_a[0] == st_m[0]
        if st_a[0] == 0:
            assert abs(ll_a[0] - ll_m[0]) <= 1e-12 * abs(ll_a[0])
        ll_all, st_all = res[11]
        if st_all[i] == 0:
            assert abs(ll_all[i] - ll_a[0]) <= 1e-12 * abs(ll_a[0])
    ll_b, st_b = res[6]
    if alone_bb[1][0] == 0:
        assert abs(ll_b[0] - alone_bb[0][0]) <= 1e-12 * abs(alone_bb[0][0])
    assert srv.stats.vectors >= 6 + 5 + 6
    lat = srv.latency_percentiles()
    assert lat is not None and lat["p99_ms"] >= lat["p50_ms"] > 0
