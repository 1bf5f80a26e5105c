"""Request server: the admission rule on CPU; alone-vs-mix equality, admission by footprint and
parity with the single-context path on the GPU."""
import numpy as np
import pytest

from acoustic_reliefs_gb300 import _lib as L
from acoustic_reliefs_gb300 import meshes
from acoustic_reliefs_gb300.serve import Server, admit_next

from tests import cases


# ------------------------------------------------------------------------------------------------
# admission rule (pure host logic)
# ------------------------------------------------------------------------------------------------
def test_admit_next_rule():
    assert admit_next([], [], 100, 0, 0) == -1
    assert admit_next([50, 10], [0, 0], 100, 0, 0) == 0          # head fits
    assert admit_next([80, 10], [0, 0], 100, 30, 1) == 1         # head does not fit, the next does
    assert admit_next([80, 90], [0, 0], 100, 30, 1) == -1        # nothing fits
    assert admit_next([80, 10], [L.SERVE_MAX_BYPASS, 0], 100, 30, 1) == -1  # head overtaken too often
    assert admit_next([120, 10], [0, 0], 100, 0, 0) == 0         # alone on an idle device it starts


def test_admission_simulation_never_starves():
    """Discrete-time run of the rule: random footprints and durations, every request starts, and
    no request is overtaken more than SERVE_MAX_BYPASS times."""
    rng = np.random.default_rng(0)
    budget = 100
    fp = rng.integers(5, 90, size=300)
    dur = rng.integers(1, 6, size=300)
    queue = list(range(300))
    bypass = {i: 0 for i in queue}
    running = {}  # id -> finish time
    started = {}
    t = 0
    while queue or running:
        for i in [i for i, f in running.items() if f <= t]:
            del running[i]
        while queue and len(running) < 4:
            in_use = sum(fp[i] for i in running)
            j = admit_next([fp[i] for i in queue], [bypass[i] for i in queue], budget, in_use, len(running))
            if j < 0:
                break
            for i in queue[:j]:
                bypass[i] += 1
            r = queue.pop(j)
            running[r] = t + dur[r]
            started[r] = t
            assert sum(fp[i] for i in running) <= budget or len(running) == 1
        t += 1
        assert t < 10000
    assert len(started) == 300
    assert max(bypass.values()) <= L.SERVE_MAX_BYPASS


# ------------------------------------------------------------------------------------------------
# GPU
# ------------------------------------------------------------------------------------------------
def _meshes():
    A = cases.relief_small()
    B = meshes.relief(0.3, 0.3, 0.05, 16, 4, 16, 0, meshes.smooth_heightmap(32, 3))
    Ps, Es = meshes.icosphere(3, 0.5)
    return [(A["Ps"], A["Es"]), (B.Ps, B.Es), (Ps, Es)]


# (mesh, frequency, incident)
_REQUESTS = [
    (0, 2000.0, ("plane", (0.0, -1.0, 0.0))),
    (1, 3000.0, ("plane", (0.3, -1.0, 0.1))),
    (2, 500.0, ("plane", (0.0, 0.0, -1.0))),
    (0, 1000.0, ("plane", (0.5, -1.0, 0.0))),
    (1, 1500.0, ("point", (0.0, 5.0, 0.0))),
    (2, 800.0, ("plane", (1.0, 0.0, 0.0))),
    (0, 2000.0, ("plane", (0.0, -1.0, 0.0))),  # the first request again
]


def _register(srv):
    return [srv.add_mesh(P, E, 32, 2.0, 1e-4, 1e-6)[0] for P, E in _meshes()]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_results_same_alone_and_in_the_mix(gpu_lib, precision):
    """Each request solved alone (one slot, one request at a time) and in a mix of seven on three
    slots gives the same pressures. Tolerance 1e-12 relative L2; every sum has a fixed order, so
    the results are expected to be bitwise equal."""
    Ls = meshes.semicircle(5.0, 181)
    alone = []
    with Server(slots=1, precision=precision) as srv:
        ids = _register(srv)
        for m, f, inc in _REQUESTS:
            y, info = srv.wait(srv.submit(ids[m], f, Ls, inc))
            assert info["status"] == 0 and info["rel_residual"] <= 1e-6
            alone.append(y)
    with Server(slots=3, precision=precision) as srv:
        ids = _register(srv)
        reqs = [srv.submit(ids[m], f, Ls, inc) for m, f, inc in _REQUESTS]
        res = [srv.wait(r) for r in reqs]
    for (y, info), ya in zip(res, alone):
        assert info["status"] == 0
        assert cases.rel_l2(y, ya) <= 1e-12
    assert cases.rel_l2(res[0][0], res[-1][0]) <= 1e-12
    # the mix really overlapped: some request started before an earlier-started one finished
    spans = sorted((i["queue_ms"], i["latency_ms"]) for _, i in res)
    assert any(spans[j + 1][0] < spans[j][1] for j in range(len(spans) - 1))
    assert len({i["slot"] for _, i in res}) > 1


@pytest.mark.gpu
def test_server_matches_diffbem_pvals(gpu_lib):
    from acoustic_reliefs_gb300.acoustics3d import DiffBEM
    c = cases.relief_small()
    bem = DiffBEM(32, 2.0, [2000.0], 1, 1e-4, 1e-4, 1e-6, precision="mixed", incident=("plane", c["vec"]))
    bem.silent = True
    bem.set_mesh(c["Ps"], c["Es"])
    y_ref = bem.pvals(2000.0, c["Ls"])
    with Server(slots=2) as srv:
        mid, _ = srv.add_mesh(c["Ps"], c["Es"], 32, 2.0, 1e-4, 1e-6)
        y, info = srv.wait(srv.submit(mid, 2000.0, c["Ls"], ("plane", c["vec"])))
    assert cases.rel_l2(y, y_ref) <= 1e-12
    assert info["iterations"] > 0 and info["hmat_bytes"] > 0


@pytest.mark.gpu
def test_admission_by_footprint_serialises(gpu_lib):
    """With a budget that holds one request's footprint but not two, requests run one at a time."""
    c = cases.relief_small()
    with Server(slots=3) as srv:
        mid, _ = srv.add_mesh(c["Ps"], c["Es"])
        _, info = srv.wait(srv.submit(mid, 2000.0, c["Ls"]))
        fp = info["footprint_bytes"]
    with Server(slots=3, hbm_budget=int(1.5 * fp)) as srv:
        mid, _ = srv.add_mesh(c["Ps"], c["Es"])
        srv.wait(srv.submit(mid, 2000.0, c["Ls"]))  # same estimate state as above
        reqs = [srv.submit(mid, 2000.0, c["Ls"]) for _ in range(3)]
        res = [srv.wait(r)[1] for r in reqs]
    spans = sorted((i["queue_ms"], i["latency_ms"]) for i in res)
    for a, b in zip(spans, spans[1:]):
        assert b[0] >= a[1] - 0.05  # next admitted only after the previous finished (clock granularity)


@pytest.mark.gpu
def test_server_rejects_oversize_and_bad_handles(gpu_lib):
    c = cases.relief_small()
    with Server(slots=1, hbm_budget=1 << 20) as srv:
        mid, _ = srv.add_mesh(c["Ps"], c["Es"])
        with pytest.raises(L.AC3DError) as e:
            srv.submit(mid, 2000.0, c["Ls"])
        assert e.value.code == L.ERR_RESOURCE
        with pytest.raises(L.AC3DError):
            srv.submit(mid + 5, 2000.0, c["Ls"])
        with pytest.raises(L.AC3DError):
            srv.poll(12345)
