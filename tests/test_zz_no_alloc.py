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
