"""CPU checks of the batched form's host side: the seeded uneven-instance
workload and argument checks of mg_batch_* (no device work)."""
import ctypes as C

import numpy as np

from mocca_gb300 import _abi, synthetic


def test_uneven_instances_workload():
    """The batched workload's seeded instances stay within the configured
    ranges and every HFB block fits the eigensolver (N <= 128)."""
    inst = synthetic.uneven_instances()
    assert len(inst) == 64
    for d in inst:
        p = d["params"]
        assert 12 <= p.nx <= 28 and p.nx == p.ny == p.nz
        assert 8 <= p.neutrons <= 40 and 8 <= p.protons <= 40
        assert p.neutrons % 2 == 0 and p.protons % 2 == 0
        assert 20 <= p.nwt <= 200 and p.nwt % 2 == 0
        assert -0.3 <= d["beta2"] <= 0.5
        nn = d["n_neutron"]
        assert nn >= p.neutrons / 2 and p.nwt - nn >= p.protons / 2
        _, qn, _ = synthetic.ho_basis(p, nn, seed=d["seed"])
        for iso in (-1, 1):
            for par in (-1, 1):
                h = int(np.sum((qn[:, 0] == iso) & (qn[:, 1] == par)))
                assert 2 * h <= 128


def test_batch_rejects_empty():
    lib = _abi.load()
    h = C.c_void_p()
    assert lib.mg_batch_create(0, None, C.byref(h)) == _abi.MG_ERR_ARG
    assert not h.value
