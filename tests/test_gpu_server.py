"""GPU: the serving loop.  Each request's result is the same alone and in
the mix; requests that arrive while others run are admitted and finish
while those still run; the memory budget bounds what runs at once."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OPTS = "gb=5, cut=999.0, rgbmax=20.0, nsnb=5, dt=0.001, gamma_ln=5.0, temp0=300.0"


def requests():
    from nabc_gb300 import sff
    out = []
    for k, (n, kind, steps) in enumerate([(300, "minimize", 60), (1200, "md", 25), (700, "minimize", 40),
                                          (2500, "minimize", 30), (500, "md", 40), (900, "minimize", 80)]):
        prm, x, _ = sff.synth_molecule(n, 500 + k)
        out.append((prm, x, kind, steps))
    return out


def test_alone_and_mixed_results_identical(lib):
    from nabc_gb300.server import Server
    reqs = requests()
    alone = []
    for prm, x, kind, steps in reqs:
        s = Server(OPTS, memory_budget_gb=20.0, max_groups=4)
        rid = s.submit(prm, x, kind, steps, 0.05)
        s.run(turns=7)
        alone.append(s.result(rid))
        s.close()
    s = Server(OPTS, memory_budget_gb=20.0, max_groups=4)
    ids = [s.submit(prm, x, kind, steps, 0.05) for prm, x, kind, steps in reqs]
    s.run(turns=7)
    for rid, a in zip(ids, alone):
        r = s.result(rid)
        assert r["status"] == a["status"]
        assert r["energy"] == a["energy"]
        assert np.array_equal(r["x"], a["x"])
    assert s.device_bytes() == 0
    s.close()


def test_continuous_admission_and_budget(lib):
    """A request that arrives while a long one runs is admitted into its own
    group and ends first; with a budget that holds one request at a time,
    the others wait and all still end."""
    from nabc_gb300 import sff
    from nabc_gb300.server import Server
    big, xb, _ = sff.synth_molecule(4000, 901)
    small, xs, _ = sff.synth_molecule(400, 902)
    s = Server(OPTS, memory_budget_gb=20.0, max_groups=4)
    a = s.submit(big, xb, "md", 200)
    nr, npend = s.pump(5)
    assert nr == 1 and npend == 0 and s.result(a) is None
    b = s.submit(small, xs, "md", 10)
    nr, npend = s.pump(5)
    assert nr == 2  # the newcomer runs beside the first request
    # each pump returns once some group's turns have run: the small request
    # (2 launches of 5 steps) ends while the large one (40) still runs
    for _ in range(10):
        if s.result(b) is not None:
            break
        s.pump(5)
    assert s.result(b) is not None and s.result(a) is None
    s.run(turns=20)
    assert s.result(a)["status"] == 200
    s.close()
    # a budget that fits only one of these requests at a time
    s = Server(OPTS, memory_budget_gb=0.008, max_groups=4)
    ids = [s.submit(small, xs + 0.01 * k, "minimize", 20, 0.05) for k in range(3)]
    nr, npend = s.pump(5)
    assert nr == 1 and npend == 2
    s.run(turns=5)
    assert all(s.result(i) is not None for i in ids)
    s.close()


def test_arrivals_join_a_running_group(lib):
    """Slot-level admission: minimisations that arrive while others run join
    that group's batch at the group's next turn that is a multiple of nsnb
    (the running systems move into a new batch with the newcomers; those
    that ended stay behind).  Every result is the same as alone, and one
    group serves them all."""
    from nabc_gb300 import sff
    from nabc_gb300.server import Server
    mols = [sff.synth_molecule(n, 700 + n) for n in (300, 700, 450, 5000, 900)]
    steps = [12, 90, 70, 60, 40]  # the first ends before the later ones join
    alone = []
    for (prm, x, _), n in zip(mols, steps):
        s = Server(OPTS, memory_budget_gb=20.0, max_groups=4)
        rid = s.submit(prm, x, "minimize", n, 0.01)
        s.run(turns=3)
        alone.append(s.result(rid))
        s.close()
    s = Server(OPTS, memory_budget_gb=20.0, max_groups=4)
    ids = []
    for k, ((prm, x, _), n) in enumerate(zip(mols, steps)):
        ids.append(s.submit(prm, x, "minimize", n, 0.01))
        for _ in range(k + 2):  # the group stops at turns 3, 5, 8, 10, ... between arrivals
            nr, npend = s.pump(3)
            assert nr <= 1
    s.run(turns=3)
    for rid, a in zip(ids, alone):
        r = s.result(rid)
        assert r["status"] == a["status"]
        assert r["energy"] == a["energy"]
        assert np.array_equal(r["x"], a["x"])
    c = s.counts()
    assert (c["groups_started"], c["joins"], c["joined_requests"]) == (1, 4, 4)
    assert s.device_bytes() == 0
    s.close()


def test_size_classes_run_apart(lib):
    """With sffg_serve_classes=1 a minimisation of another size class (4,096
    atoms and up) starts its own group beside the running one instead of
    joining it; results as alone."""
    from nabc_gb300 import sff
    from nabc_gb300.server import Server
    small, xs, _ = sff.synth_molecule(400, 811)
    big, xb, _ = sff.synth_molecule(4200, 812)
    opts = OPTS + ", sffg_serve_classes=1"
    alone = []
    for prm, x in ((small, xs), (big, xb)):
        s = Server(opts, memory_budget_gb=20.0, max_groups=4)
        rid = s.submit(prm, x, "minimize", 30, 0.01)
        s.run(turns=4)
        alone.append(s.result(rid))
        s.close()
    s = Server(opts, memory_budget_gb=20.0, max_groups=4)
    a = s.submit(small, xs, "minimize", 30, 0.01)
    s.pump(4)
    b = s.submit(big, xb, "minimize", 30, 0.01)
    nr, _ = s.pump(4)
    assert nr == 2
    s.run(turns=4)
    for rid, r0 in zip((a, b), alone):
        r = s.result(rid)
        assert (r["status"], r["energy"]) == (r0["status"], r0["energy"])
        assert np.array_equal(r["x"], r0["x"])
    s.close()
