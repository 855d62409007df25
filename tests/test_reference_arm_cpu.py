"""The CPU side of the bench's reference arm (no GPU): the oracle and the host-built setup map no
engine library, the oracle's own config defaults equal the engine's, and bonds built on the host
cores in one pass equal scipy's query_pairs per particle."""
import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np

from peridem_gb300 import gen

ROOT = Path(__file__).resolve().parent.parent


def test_oracle_and_host_setup_map_no_engine_library():
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "from peridem_gb300 import gen\n"
        "from oracle import oracle as O\n"
        "gen.set_bond_builder('cpu')\n"
        "s, cfg = gen.crush512(n=2, count=3)\n"
        "o = O.Oracle(s, cfg, threads=2)\n"
        "o.step(2)\n"
        "assert o.counts()['live_bonds'] > 0\n"
        "o.close()\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert 'libpd_oracle' in maps\n"
        "assert 'libperidem_gb300' not in maps, 'the engine library was mapped'\n"
        "print('ok')\n" % str(ROOT))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr


def test_oracle_config_defaults_equal_the_engine_defaults():
    from oracle import oracle as O
    from peridem_gb300 import _capi
    a = O.default_config()
    b = _capi.default_config()
    assert C.string_at(C.addressof(a), C.sizeof(a)) == C.string_at(C.addressof(b), C.sizeof(b))
    c = O.default_config(dt=1e-9, self_contact=0)
    assert c.dt == 1e-9 and c.self_contact == 0


def test_deferred_host_bonds_equal_query_pairs_per_particle():
    from scipy.spatial import cKDTree
    gen.set_bond_builder("cpu")
    s, _ = gen.crush512(n=2)
    for p in range(s.n_particles):
        sl = s.particle_slice(p)
        pr = cKDTree(s.pos[sl]).query_pairs(float(s.delta[p]), output_type="ndarray")
        want = pr[np.lexsort((pr[:, 1], pr[:, 0]))].astype(np.uint32)
        np.testing.assert_array_equal(s.particle_conn(p), want, err_msg=f"particle {p}")
