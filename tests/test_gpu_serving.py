"""Serving loop: each result is the same alone and in the mix, agrees with the
plain per-call complex128 path, and admission by HBM footprint evicts idle
clients without changing results.

Tolerances: complex64 served <H> against the complex128 plain path within
1e-5 * sum|coef| (float32 rounding of a depth <= 6 ansatz); alone vs mix within
1e-6 relative (the same passes, possibly on the generic or the specialised
kernel while the tiered compile finishes)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def specs(seed=5):
    from bluetangle_gpu.serving import make_client
    rng = np.random.default_rng(seed)
    out = []
    kinds = [("sv", 11, 4), ("sv", 14, 5), ("sv", 9, 3), ("traj", 6, 3), ("dm", 5, 3), ("sv", 16, 6)]
    for cid, (kind, n, depth) in enumerate(kinds):
        c = make_client(rng, cid, kind, n, depth)
        c.ntraj = 8
        out.append(c)
    return out


def requests(sp, per_client=3, seed=9):
    from bluetangle_gpu.serving import Request
    rng = np.random.default_rng(seed)
    reqs = []
    rid = 0
    for r in range(per_client):
        for s in sp:
            reqs.append(Request(rid, s.cid, rng.normal(0, 0.3, s.nparams), seed=1000 + rid))
            rid += 1
    return reqs


def test_results_alone_equal_in_mix(ctx):
    import bluetangle_gpu.serving as S
    sp = specs()
    alone = {}
    srv = S.Server(sp, lanes=1)
    try:
        for req in requests(sp):
            srv.submit(req)
            req.done.wait(120)
            assert req.error is None, req.error
            alone[req.rid] = req.value
    finally:
        srv.close()
    srv = S.Server(sp, lanes=4)
    try:
        reqs = requests(sp)
        for req in reqs:
            srv.submit(req)
        for req in reqs:
            req.done.wait(120)
            assert req.error is None, req.error
    finally:
        srv.close()
    for req in reqs:
        a = alone[req.rid]
        assert abs(req.value - a) <= 1e-6 * max(1.0, abs(a)), (req.cid, req.value, a)
    lat = np.array([r.t_done - r.t_submit for r in reqs])
    assert np.all(lat > 0)


def test_served_values_match_plain_complex128(ctx):
    import bluetangle_gpu as bt
    import bluetangle_gpu.serving as S
    sp = specs(7)
    reqs = requests(sp, per_client=1, seed=13)
    srv = S.Server(sp, lanes=3)
    try:
        for req in reqs:
            srv.submit(req)
        for req in reqs:
            req.done.wait(120)
            assert req.error is None, req.error
    finally:
        srv.close()
    pctx = bt.Context(0, seed=3)
    try:
        for req in reqs:
            spec = sp[req.cid]
            ref = S.plain_request(spec, req.theta, req.seed, pctx, prec="c128")
            scale = sum(abs(t[0]) for t in spec.terms)
            assert abs(req.value - ref) < 1e-5 * scale, (spec.kind, spec.n, req.value, ref)
    finally:
        pctx.close()


def test_admission_evicts_idle_clients(ctx):
    import bluetangle_gpu.serving as S
    sp = specs(11)
    budget = max(s.footprint("c64") for s in sp) * 2  # room for about two clients at a time
    reqs = requests(sp, per_client=2, seed=17)
    srv = S.Server(sp, lanes=2, hbm_budget=budget)
    try:
        for req in reqs:
            srv.submit(req)
        for req in reqs:
            req.done.wait(120)
            assert req.error is None, req.error
        assert srv.used <= budget
    finally:
        srv.close()
    alone = S.Server(sp, lanes=1)
    try:
        for req in requests(sp, per_client=2, seed=17):
            alone.submit(req)
            req.done.wait(120)
            match = [r for r in reqs if r.rid == req.rid][0]
            assert abs(match.value - req.value) <= 1e-6 * max(1.0, abs(req.value))
    finally:
        alone.close()


def test_native_server_alone_equals_mix_and_python_server(ctx):
    """The library's serving engine (bt_serve_*): each result is the same served
    alone (one lane, one request at a time) and in the mix (4 lanes, all requests
    queued at once), and plan clients agree with the Python server (same passes)."""
    import bluetangle_gpu.serving as S
    sp = specs(21)
    alone = {}
    srv = S.NativeServer(sp, lanes=1)
    try:
        for req in requests(sp, per_client=2, seed=23):
            srv.submit(req)
            srv.wait(req)
            assert req.error is None, req.error
            alone[req.rid] = req.value
    finally:
        srv.close()
    srv = S.NativeServer(sp, lanes=4)
    try:
        reqs = requests(sp, per_client=2, seed=23)
        for req in reqs:
            srv.submit(req)
        for req in reqs:
            srv.wait(req)
            assert req.error is None, req.error
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["p99_s"] >= st["p50_s"] > 0
    finally:
        srv.close()
    for req in reqs:
        a = alone[req.rid]
        assert abs(req.value - a) <= 1e-6 * max(1.0, abs(a)), (req.cid, req.value, a)
    py = S.Server(sp, lanes=2)
    try:
        preqs = [r for r in requests(sp, per_client=2, seed=23) if sp[r.cid].kind != "traj"]
        for req in preqs:
            py.submit(req)
        for req in preqs:
            req.done.wait(120)
            assert req.error is None, req.error
            s = sp[req.cid]
            if s.kind == "sv" and s.footprint("c64", pack=8) > s.footprint("c64"):
                # packed client: a program (one CTA per request) against the Python
                # server's fused plan, both complex64: within complex64 accuracy
                tol = 2e-5 * sum(abs(t[0]) for t in s.terms)
            else:
                tol = 1e-6 * max(1.0, abs(req.value))
            assert abs(req.value - alone[req.rid]) <= tol, (req.cid, req.value)
    finally:
        py.close()


def test_native_server_packs_small_circuits_into_one_launch(ctx):
    """Eight requests of one small state-vector client queued at once run as one
    packed program launch (they finish together) and each equals its value served
    alone, and its complex128 plain-path value within complex64 accuracy."""
    import bluetangle_gpu.serving as S
    sp = specs(37)[:1]  # sv, 11 qubits
    reqs = requests(sp, per_client=8, seed=41)
    srv = S.NativeServer(sp, lanes=1, pack=8)
    try:
        for req in reqs:
            srv.submit(req)
        for req in reqs:
            srv.wait(req)
            assert req.error is None, req.error
        st = srv.stats()
    finally:
        srv.close()
    assert st["completed"] == len(reqs) and st["runs"] < len(reqs)  # requests shared launches
    one = S.NativeServer(sp, lanes=1, pack=8)
    pctx = S.Context(0, seed=3)
    try:
        for r in requests(sp, per_client=8, seed=41):
            one.submit(r)
            one.wait(r)
            match = [q for q in reqs if q.rid == r.rid][0]
            assert abs(match.value - r.value) <= 1e-6 * max(1.0, abs(r.value))
            ref = S.plain_request(sp[0], r.theta, r.seed, pctx, prec="c128")
            assert abs(r.value - ref) <= 2e-5 * sum(abs(t[0]) for t in sp[0].terms)
    finally:
        one.close()
        pctx.close()


def test_native_server_admission_by_footprint(ctx):
    """With room for about two clients, the engine evicts idle residents and every
    request still completes with the value it has alone."""
    import bluetangle_gpu.serving as S
    sp = specs(29)
    budget = max(s.footprint("c64", pack=8) for s in sp) * 2
    srv = S.NativeServer(sp, lanes=2, hbm_budget=budget)
    try:
        reqs = requests(sp, per_client=2, seed=31)
        for req in reqs:
            srv.submit(req)
        for req in reqs:
            srv.wait(req)
            assert req.error is None, req.error
        st = srv.stats()
        assert st["hbm_used"] <= budget and st["resident"] <= len(sp)
    finally:
        srv.close()
    one = S.NativeServer(sp, lanes=1)
    try:
        for req in requests(sp, per_client=2, seed=31):
            one.submit(req)
            one.wait(req)
            match = [r for r in reqs if r.rid == req.rid][0]
            assert abs(match.value - req.value) <= 1e-6 * max(1.0, abs(req.value))
    finally:
        one.close()


def test_native_server_runs_queued_plan_requests_together(ctx):
    """A plan client of 16 qubits (a state too small to fill the GPU) holds 8
    members: eight of its requests queued at once run as one plan run over the
    members, each with its own matrices, and each equals its value served alone."""
    import bluetangle_gpu.serving as S
    sp = specs(43)[5:6]  # sv, 16 qubits: a fused plan
    reqs = requests(sp, per_client=8, seed=47)
    srv = S.NativeServer(sp, lanes=1)
    try:
        for req in reqs:
            srv.submit(req)
        for req in reqs:
            srv.wait(req)
            assert req.error is None, req.error
        st = srv.stats()
    finally:
        srv.close()
    assert st["completed"] == len(reqs) and st["runs"] < len(reqs)  # requests shared plan runs
    one = S.NativeServer(sp, lanes=1)
    try:
        for r in requests(sp, per_client=8, seed=47):
            one.submit(r)
            one.wait(r)
            match = [q for q in reqs if q.rid == r.rid][0]
            assert abs(match.value - r.value) <= 1e-6 * max(1.0, abs(r.value)), (match.value, r.value)
    finally:
        one.close()
