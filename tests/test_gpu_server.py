"""Request server (ommp_gpu_server_*): a request's result must not depend on
what else is running.  Each system is solved alone through OMMPSystem (a new
field from a cold start, then a follow-up field warm-started from the first
dipoles) and again through the server with every request in flight at once,
under a budget large enough for all systems and under one so small that
systems are evicted and re-admitted.  FP64 results agree to 1e-9 (relative),
mixed ones to 1e-7; the admission bookkeeping never exceeds the budget.
"""
import numpy as np
import pytest

from openmmpol_gb300 import OMMPError, OMMPSystem, Server, kernel_launch_count, set_verbose, synth

pytestmark = pytest.mark.gpu

SIZES = [40, 120, 260, 700, 900]


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


@pytest.fixture(scope="module", autouse=True)
def quiet():
    set_verbose(0)


@pytest.fixture(scope="module")
def systems(tmp_path_factory):
    d = tmp_path_factory.mktemp("srv")
    out = []
    for k, n in enumerate(SIZES):
        w = synth.water_cluster(n, seed=20 + k)
        path = synth.write_mmp(str(d / f"w{n}.mmp"), w)
        g = OMMPSystem(path)
        rng = np.random.default_rng(k)
        f0 = rng.standard_normal((g.pol_atoms, 3)) * 1e-3
        f1 = f0 * (1 + 0.01 * rng.standard_normal((g.pol_atoms, 3)))
        out.append({"path": path, "n": g.pol_atoms, "nipd": g.n_ipd, "fields": (f0, f1)})
        g.close()
    return out


def alone(sysd, precision):
    g = OMMPSystem(sysd["path"])
    g.set_precision(precision)
    g.set_solver_tol(1e-10)
    res = []
    for f in sysd["fields"]:
        g.set_external_field(f)  # the second call warm-starts from the first dipoles
        res.append((g.ipd, g.get_polelec_energy()))
    g.close()
    return res


def served(server, systems):
    """All new requests in flight together, then all follow-ups together."""
    rids = [server.submit(s["path"], s["fields"][0], s["nipd"]) for s in systems]
    first = [server.wait(r) for r in rids]
    rids = [server.submit_followup(o["instance"], s["fields"][1], s["nipd"]) for o, s in zip(first, systems)]
    second = [server.wait(r) for r in rids]
    return first, second


def check(systems, first, second, precision):
    tol = 1e-9 if precision == "fp64" else 1e-7
    for s, a, b in zip(systems, first, second):
        ref = alone(s, precision)
        assert rel(a["ipd"], ref[0][0]) < tol
        assert abs(a["energy"] - ref[0][1]) < tol * abs(ref[0][1])
        assert rel(b["ipd"], ref[1][0]) < tol
        assert abs(b["energy"] - ref[1][1]) < tol * abs(ref[1][1])
        assert a["latency_ms"] > 0 and b["latency_ms"] > 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_results_same_alone_and_in_the_mix(systems, precision):
    srv = Server(8 << 30, slots=4, precision=precision, tol=1e-10)
    l0 = kernel_launch_count()
    first, second = served(srv, systems)
    launched = kernel_launch_count() - l0
    st = srv.stats()
    ph = srv.phase_stats()
    srv.close()
    check(systems, first, second, precision)
    # where the new systems' latency went: every phase accounted, the sum
    # within the mean latency of the new requests
    assert ph["new_systems"] == len(systems)
    phases = [ph[k] for k in ("queue_ms", "host_setup_ms", "admission_ms", "upload_ms", "field_ms", "solve_ms")]
    assert min(phases) >= 0.0 and ph["host_setup_ms"] > 0.0 and ph["solve_ms"] > 0.0
    assert (ph["field_ms"] > 0.0) == (precision != "fp64")
    mean_new = np.mean([a["latency_ms"] for a in first])
    assert sum(phases) <= mean_new * 1.01 + 1.0
    # the launch count stays exact while solves on several threads capture
    # and replay CUDA graphs (10 solves of at most a few hundred kernels)
    assert 0 < launched < 20000
    for a, b in zip(first, second):
        assert a["instance"] == b["instance"]  # follow-ups reuse the resident system
    assert st["evictions"] == 0 and st["resident"] == len(systems)
    assert st["completed"] == 2 * len(systems)
    assert st["peak_concurrent"] >= 2


def test_engine_serves_uneven_systems_in_shared_launches(systems):
    """In the mixed modes the server's solves run in the multi-system
    engine: systems of 120 to 2,700 sites in flight together share product
    launches, and each result still equals its solve alone."""
    srv = Server(8 << 30, slots=len(systems), precision="mixed-ds", tol=1e-10)
    with pytest.raises(OMMPError):
        srv.set_round_ms(-1.0)
    srv.set_round_ms(1.0)  # short rounds: more of them, same results
    first, second = served(srv, systems)
    es = srv.engine_stats()
    srv.close()
    check(systems, first, second, "mixed-ds")
    assert es["max_systems_per_launch"] >= 2 and es["shared_launches"] >= 1
    assert es["rounds"] > 0 and es["launches"] >= es["shared_launches"]
    # the rounds' time: GPU time of products and bookkeeping within the rounds' wall time
    assert es["product_gpu_ms"] > 0.0 and es["bookkeeping_gpu_ms"] > 0.0
    assert es["round_wall_ms"] >= es["product_gpu_ms"]


def test_eviction_under_small_budget(systems):
    # size every system on the device, then give room for the largest two only
    srv = Server(8 << 30, slots=1, precision="mixed", tol=1e-10)
    need = []
    for s in systems:
        o = srv.wait(srv.submit(s["path"], s["fields"][0], s["nipd"]))
        before = srv.stats()["bytes_in_use"]
        srv.release(o["instance"])
        need.append(before - sum(need))
    srv.close()
    budget = int(sorted(need)[-1] + sorted(need)[-2] + 1)

    srv = Server(budget, slots=3, precision="mixed", tol=1e-10)
    rids = [srv.submit(s["path"], s["fields"][0], s["nipd"]) for s in systems]
    first = [srv.wait(r) for r in rids]
    second = []
    for o, s in zip(first, systems):
        try:
            r = srv.submit_followup(o["instance"], s["fields"][1], s["nipd"])
            second.append(srv.wait(r))
        except OMMPError:
            # evicted since: resubmit the system and replay its history
            o2 = srv.wait(srv.submit(s["path"], s["fields"][0], s["nipd"]))
            second.append(srv.wait(srv.submit_followup(o2["instance"], s["fields"][1], s["nipd"])))
    st = srv.stats()
    srv.close()
    check(systems, first, second, "mixed")
    assert st["evictions"] >= 1
    assert st["peak_bytes"] <= budget


def test_cancel_queued_request(systems):
    big, small = systems[-1], systems[0]
    srv = Server(8 << 30, slots=1, precision="fp64", tol=1e-10)
    r1 = srv.submit(big["path"], big["fields"][0], big["nipd"])
    r2 = srv.submit(small["path"], small["fields"][0], small["nipd"])
    assert srv.cancel(r2)  # one slot, busy with r1 for far longer than this call
    with pytest.raises(OMMPError) as e:
        srv.wait(r2)
    assert e.value.status == 7
    o = srv.wait(r1)
    assert not srv.cancel(r1)  # done
    srv.close()
    ref = alone(big, "fp64")
    assert rel(o["ipd"], ref[0][0]) < 1e-9


def test_errors(systems, tmp_path):
    s = systems[0]
    srv = Server(1 << 20, slots=2, precision="mixed")  # 1 MiB: nothing fits
    with pytest.raises(OMMPError):
        srv.wait(srv.submit(s["path"], s["fields"][0], s["nipd"]))
    srv.close()
    srv = Server(1 << 30, slots=2, precision="mixed")
    with pytest.raises(OMMPError):
        srv.wait(srv.submit(str(tmp_path / "missing.mmp"), s["fields"][0], s["nipd"]))
    with pytest.raises(OMMPError):
        srv.wait(srv.submit_followup(12345, s["fields"][0], s["nipd"]))
    o = srv.wait(srv.submit(s["path"], s["fields"][0], s["nipd"]))
    with pytest.raises(OMMPError):  # field of the wrong size
        srv.wait(srv.submit_followup(o["instance"], s["fields"][0][:-1], s["nipd"]))
    srv.close()
