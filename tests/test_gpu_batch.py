"""GPU checks of the batched form: independent instances of uneven mesh
size, spwf count and particle number, each with a Q20 constraint, run
concurrently by mg_batch_* give the same results as each instance run on
its own (the kernels are deterministic: fixed-order reductions), and the
schedule autotuner picks a valid worker count."""
import numpy as np
import pytest

from mocca_gb300 import SLY4, _abi, synthetic
from mocca_gb300.mesh import Batch, MeshState

pytestmark = pytest.mark.gpu


def _instances(count, seed=11):
    return synthetic.uneven_instances(count, seed=seed, n_range=(10, 14))


def _state(d):
    p = d["params"]
    psi, qn, en = synthetic.ho_basis(p, d["n_neutron"], seed=d["seed"])
    g = MeshState(p, SLY4)
    g.set_spinors(psi, qn)
    g.set_energies(en)
    g.set_pairing()
    g.add_constraint(2, 0, d["q20"])
    g.Start()
    return g


def test_batch_matches_instances_run_alone(built):
    inst = _instances(5)
    alone = []
    for d in inst:
        g = _state(d)
        alone.append(g.Evolve(3, 0.010, 0.3)["total"])
        g.close()
    states = [_state(d) for d in inst]
    b = Batch(states)
    assert b.set_workers(3) == 3
    out = b.Evolve(3, 0.010, 0.3)
    for e_b, e_a in zip([o["total"] for o in out], alone):
        assert np.isfinite(e_b)
        assert abs(e_b - e_a) <= 1e-10 * max(1.0, abs(e_a)), (e_b, e_a)
    b.close()
    for s in states:
        s.close()


def test_batch_tune_and_continue(built):
    inst = _instances(6, seed=12)
    states = [_state(d) for d in inst]
    b = Batch(states)
    w = b.tune(1, 0.010, 0.3)
    assert 1 <= w <= len(states)
    out = b.Evolve(2, 0.010, 0.3)
    assert all(np.isfinite(o["total"]) for o in out)
    # the constraint pulls each instance's Q20 towards its target
    for s, d in zip(states, inst):
        st = s.get_constraint(0)
        assert st["active"]
    b.close()
    for s in states:
        s.close()


def test_batch_failed_instance_is_skipped(built):
    """An instance that fails (here: no spinors were ever uploaded, which the
    library reports as MG_ERR_STATE before any device work) is marked failed
    and skipped; the other instances of the batch carry on unchanged."""
    inst = _instances(3, seed=13)
    alone = []
    for d in (inst[0], inst[2]):
        g = _state(d)
        alone.append(g.Evolve(2, 0.010, 0.3)["total"])
        g.close()
    states = [_state(inst[0]), MeshState(inst[1]["params"], SLY4), _state(inst[2])]
    b = Batch(states)
    b.set_workers(2)
    out = b.Evolve(2, 0.010, 0.3, allow_failures=True)
    st = b.status()
    assert st[1] == _abi.MG_ERR_STATE and st[0] >= 0 and st[2] >= 0
    for e_b, e_a in zip((out[0]["total"], out[2]["total"]), alone):
        assert abs(e_b - e_a) <= 1e-10 * max(1.0, abs(e_a)), (e_b, e_a)
    # later calls skip it and report the healthy instances' status
    out = b.Evolve(1, 0.010, 0.3)
    assert np.isfinite(out[0]["total"]) and np.isfinite(out[2]["total"])
    assert b.status()[1] == _abi.MG_ERR_STATE
    b.close()
    for s in states:
        s.close()


def test_batch_rejects_a_context_listed_twice(built):
    import ctypes as C
    g = _state(_instances(1, seed=13)[0])
    lib = _abi.load()
    arr = (C.c_void_p * 2)(g.h.value, g.h.value)
    h = C.c_void_p()
    assert lib.mg_batch_create(2, arr, C.byref(h)) == _abi.MG_ERR_ARG
    assert not h.value
    g.close()
