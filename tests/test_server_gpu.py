"""Request server (bem_server_*): independent solves of different meshes,
wavenumbers and source counts admitted while others run, by device
footprint, with assembled systems reused across requests that share geometry
and wavenumber.  Every result is checked against the FP64 solve of its own
system (1e-5 relative) and against the same request solved alone."""
import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu


def _chief(rng, rmax, n=8):
    u = rng.random((n, 3))
    r = rmax * np.cbrt(u[:, 0])
    th = np.arccos(1 - 2 * u[:, 1])
    ph = 2 * np.pi * u[:, 2]
    return np.stack([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)], axis=1)


def _requests(bemlib, n=8, seed=7):
    """Seeded ellipsoids (semi-axes in [0.05, 0.2] m) at icosphere
    subdivisions 1-3, 200 Hz - 4 kHz, 1-12 point sources on a 1 m sphere."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        sub = [2, 1, 3, 2][i % 4]
        ax = rng.uniform(0.05, 0.2, 3)
        m = bemlib.Mesh.icosphere(sub).perturbed_ellipsoid(*ax, lmax=4, amp=0.05, seed=100 + i)
        k = 2 * np.pi * rng.uniform(200.0, 4000.0) / 343.21
        S = int(rng.integers(1, 13))
        rot = np.linalg.qr(rng.standard_normal((3, 3)))[0]
        srcs = [("point", s, 1.0) for s in bemlib.fibonacci_sphere(S, 1.0) @ rot.T]
        out.append(dict(pnts=m.points(), elems=m.elems(), k=k, srcs=srcs,
                        chief=_chief(rng, 0.4 * ax.min())))
    return out


def _fp64(bemlib, r):
    s = bemlib.Solver()
    s.set_geometry(r["pnts"], r["elems"], chief=r["chief"])
    s.set_sources(r["srcs"])
    s.assemble(r["k"], bemlib.PREC_C128)
    s.solve(bemlib.SOLVE_QR)
    return s.solution()


def _run(server, reqs, together):
    xs, res = [None] * len(reqs), [None] * len(reqs)
    if together:
        tickets = [server.submit(r["pnts"], r["elems"], r["k"], r["srcs"], chief=r["chief"]) for r in reqs]
        for i, t in enumerate(tickets):
            xs[i], res[i] = server.wait(t)
    else:
        for i, r in enumerate(reqs):
            t = server.submit(r["pnts"], r["elems"], r["k"], r["srcs"], chief=r["chief"])
            xs[i], res[i] = server.wait(t)
    return xs, res


def test_mix_matches_alone_and_fp64(bemlib):
    reqs = _requests(bemlib)
    with bemlib.Server(slots=1, cache_systems=0) as alone:
        xa, ra = _run(alone, reqs, together=False)
        assert alone.stats()["max_in_flight"] == 1
    with bemlib.Server(slots=4, cache_systems=0) as mix:
        xm, rm = _run(mix, reqs, together=True)
        st = mix.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["max_in_flight"] >= 2, st           # requests overlapped on the device
    assert st["solves"] == sum(len(r["srcs"]) for r in reqs)
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    for i, r in enumerate(reqs):
        x64 = _fp64(bemlib, r)
        assert xm[i].shape == (r["pnts"].shape[0], len(r["srcs"]))
        assert rel_err(xm[i], x64) < 1e-5, (i, rel_err(xm[i], x64))
        assert rel_err(xm[i], xa[i]) < 1e-6, (i, rel_err(xm[i], xa[i]))
        assert rm[i]["converged"] == 1 and rm[i]["latency_ms"] >= rm[i]["service_ms"] > 0
        want = bemlib.SOLVE_BLOCK_GMRES if len(r["srcs"]) >= 4 else bemlib.SOLVE_GMRES_REFINED
        assert rm[i]["method"] == want


def test_cached_system_reused_for_new_sources(bemlib):
    r = _requests(bemlib, n=1, seed=11)[0]
    r2 = dict(r, srcs=[("point", (0.9, -0.3, 0.2), 1.0), ("plane", (0.0, 0.6, 0.8), 1.0)])
    with bemlib.Server(slots=2, cache_systems=4) as srv:
        _, res1 = srv.wait(srv.submit(r["pnts"], r["elems"], r["k"], r["srcs"], chief=r["chief"]))
        x2, res2 = srv.wait(srv.submit(r2["pnts"], r2["elems"], r2["k"], r2["srcs"], chief=r2["chief"]))
        # same geometry at another wavenumber is a different system
        _, res3 = srv.wait(srv.submit(r["pnts"], r["elems"], 1.1 * r["k"], r["srcs"], chief=r["chief"]))
        st = srv.stats()
    assert res1["cache_hit"] == 0 and res2["cache_hit"] == 1 and res3["cache_hit"] == 0
    assert st["cache_hits"] == 1
    assert rel_err(x2, _fp64(bemlib, r2)) < 1e-5


def test_admission_by_footprint(bemlib):
    reqs = _requests(bemlib, n=4, seed=5)
    big = max(reqs, key=lambda r: r["pnts"].shape[0] * len(r["srcs"]))
    with bemlib.Server(slots=1, cache_systems=0) as probe:
        _, res = probe.wait(probe.submit(big["pnts"], big["elems"], big["k"], big["srcs"], chief=big["chief"]))
    need = res["device_bytes"]
    same = [dict(big, k=big["k"] * (1 + 0.01 * i)) for i in range(4)]
    # room for one request at a time: they run one after another
    with bemlib.Server(slots=4, cache_systems=0, hbm_budget_bytes=1.5 * need) as srv:
        xs, rs = _run(srv, same, together=True)
        st = srv.stats()
        assert st["max_in_flight"] == 1 and st["completed"] == 4
        assert st["peak_bytes"] <= 1.5 * need
        # a request above the budget is refused, the server keeps serving
        with pytest.raises(bemlib.BemError) as ei:
            srv.wait(srv.submit(big["pnts"], big["elems"], big["k"], big["srcs"] * 40, chief=big["chief"]))
        assert ei.value.status == bemlib.ERR_TOO_LARGE
        x, _ = srv.wait(srv.submit(big["pnts"], big["elems"], big["k"], big["srcs"], chief=big["chief"]))
    assert rel_err(x, _fp64(bemlib, big)) < 1e-5
