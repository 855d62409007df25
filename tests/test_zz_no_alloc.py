"""pd_count_live_bonds_noalloc: the live-bond count for callers that must not allocate device
memory (a monitor polling a running simulation, where cudaMalloc would synchronise the device
under the step pipeline, or an application whose free HBM is all held by resident
simulations). Its scratch is a static device array shared by every call, so this checks that
consecutive calls agree with the allocating pd_count_live_bonds, including after the count has
changed (bonds breaking between calls), i.e. that no stale scratch leaks into a result.

The file name makes pytest collect it last; it passes alone in a fresh process as well."""
import ctypes as C

import pytest

from peridem_gb300 import _capi
from peridem_gb300.sim import Sim
from tests import cases

pytestmark = pytest.mark.gpu


def _noalloc(sim) -> int:
    n = C.c_uint64()
    rc = _capi.lib().pd_count_live_bonds_noalloc(sim.h, C.byref(n))
    assert rc == 0, _capi.lib().pd_last_error(sim.h).decode()
    return int(n.value)


def test_noalloc_live_bonds_matches_allocating_entry_point():
    s, cfg = cases.impact_free()
    sim = Sim(s, cfg, "fp64")
    sim.step(5)
    ref1 = sim.live_bonds()
    first = _noalloc(sim)
    second = _noalloc(sim)
    assert first == ref1
    assert second == ref1
    sim.step(cfg["timesteps"])  # the impact breaks bonds: the count changes
    ref2 = sim.live_bonds()
    assert ref2 < ref1
    third = _noalloc(sim)
    fourth = _noalloc(sim)
    assert third == ref2
    assert fourth == ref2
    sim.close()


def test_noalloc_fp32c_handle():
    s, cfg = cases.cubes_gravity()
    sim = Sim(s, cfg, "fp32c")
    sim.step(10)
    assert _noalloc(sim) == sim.live_bonds()
    assert _noalloc(sim) == sim.live_bonds()
    sim.close()


def test_noalloc_refuses_handles_above_its_limit():
    """A handle of more nodes than the static scratch holds (1,048,576) gets PD_EINVAL and a
    message naming the limit; the allocating entry point still counts it."""
    import numpy as np

    from peridem_gb300.setupdata import concat
    n = 102
    ax = np.arange(n) * 1e-3  # nodes 1 mm apart, horizon 0.1 mm: no bonds, no contacts
    X, Y, Z = np.meshgrid(ax, ax, ax[:101], indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    assert len(pos) > 1 << 20
    part = dict(pos=pos, vol=np.full(len(pos), 1e-12), conn=np.zeros((0, 2), np.uint32),
                rho=2440.0, delta=1e-4, cnot=1.0, snot=1e-3)
    s = concat([part], dict(contact_radius=1e-5, normal_stiffness=1.0, damping_ratio=0.8,
                            friction_coefficient=0.3), None)
    sim = Sim(s, dict(dt=1e-9, timesteps=1, enable_fracture=0), "fp64")
    n_out = C.c_uint64(12345)
    rc = _capi.lib().pd_count_live_bonds_noalloc(sim.h, C.byref(n_out))
    assert rc == _capi.PD_EINVAL
    msg = _capi.lib().pd_last_error(sim.h).decode()
    assert "1048576" in msg and str(len(pos)) in msg, msg
    assert n_out.value == 12345  # nothing written on refusal
    assert sim.live_bonds() == 0
    sim.close()
