"""GPU bond lists (pd_query_pairs) against the reference's own call, scipy's
cKDTree.query_pairs(delta) sorted (exp_dict.py:542-567), on jittered lattices of every shape,
and against the distance test itself, ((dx*dx + dy*dy) + dz*dz) <= r*r evaluated by numpy, on
points placed within a few ulps of the radius and on batches with empty and single-node sets.

scipy's compiled distance loop is platform code: x86 builds evaluate that expression as
written (checked here on 80,000 pairs within 3 ulps of r), while aarch64 builds contract it
into fused multiply-adds, which moves pairs lying within an ulp of r. Against scipy, a pair may
therefore differ only if its squared distance is within 4 ulps of r*r."""
import numpy as np
import pytest

from peridem_gb300 import gen

pytestmark = pytest.mark.gpu


def _formula(pos, r):
    """All pairs i < j with ((dx*dx + dy*dy) + dz*dz) <= r*r (numpy: no contraction), sorted."""
    n = len(pos)
    if n < 2:
        return np.zeros((0, 2), dtype=np.uint32)
    i, j = np.triu_indices(n, 1)
    d = pos[j] - pos[i]
    keep = ((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]) <= r * r
    return np.stack([i[keep], j[keep]], axis=1).astype(np.uint32)


def _same_up_to_boundary(got, ref, pos, r):
    a = {tuple(x) for x in got.tolist()}
    b = {tuple(x) for x in ref.tolist()}
    for i, j in a ^ b:
        d = pos[j] - pos[i]
        s2 = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]
        assert abs(s2 - r * r) <= 4 * np.spacing(r * r), f"pair {(i, j)} differs away from the radius"
    # order: sorted by (i, j)
    assert np.array_equal(got, got[np.lexsort((got[:, 1], got[:, 0]))]) if len(got) else True


def _cpu(pos, r):
    from scipy.spatial import cKDTree
    pr = cKDTree(pos).query_pairs(r, output_type="ndarray")
    if len(pr) == 0:
        return np.zeros((0, 2), dtype=np.uint32)
    return pr[np.lexsort((pr[:, 1], pr[:, 0]))].astype(np.uint32)


@pytest.mark.parametrize("kind,size", [("sphere", 1.0e-3), ("cube", 0.8e-3), ("ellipsoid", (1.2e-3, 0.7e-3, 0.9e-3))])
def test_lattices_equal_query_pairs(kind, size):
    rng = np.random.default_rng(5)
    h = 0.1e-3
    P = gen.lattice(kind, size, h)
    P = P @ gen.random_rotation(rng).T + rng.uniform(-0.05 * h, 0.05 * h, size=P.shape) + 0.3e-3
    got = gen.bonds_gpu([P], [3 * h])[0]
    _same_up_to_boundary(got, _cpu(P, 3 * h), P, 3 * h)
    if len(P) <= 3000:
        np.testing.assert_array_equal(got, _formula(P, 3 * h))


def test_points_at_the_radius():
    rng = np.random.default_rng(11)
    r = 3e-4
    sets, radii = [], []
    for _ in range(40):
        c = rng.uniform(-1e-3, 1e-3, 3)
        d = rng.normal(size=(300, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
        pts = c + d * r
        pts = pts + rng.integers(-3, 4, size=pts.shape) * np.spacing(np.abs(pts))
        sets.append(np.vstack([c[None, :], pts]))
        radii.append(r)
    got = gen.bonds_gpu(sets, radii)
    for P, g in zip(sets, got):
        np.testing.assert_array_equal(g, _formula(P, r))
        _same_up_to_boundary(g, _cpu(P, r), P, r)


def test_batch_with_empty_and_single_sets():
    rng = np.random.default_rng(3)
    sets = [np.zeros((0, 3)), rng.uniform(0, 1e-3, (1, 3)), rng.uniform(0, 1e-3, (500, 3)),
            np.zeros((0, 3)), rng.uniform(0, 2e-3, (800, 3))]
    radii = [1e-4, 1e-4, 2e-4, 5e-5, 3.5e-4]
    got = gen.bonds_gpu(sets, radii)
    for P, r, g in zip(sets, radii, got):
        np.testing.assert_array_equal(g, _formula(P, r))


def test_generator_setups_identical_with_gpu_builder():
    s_cpu, _ = gen.crush512(n=2)
    gen.set_bond_builder("gpu")
    try:
        s_gpu, _ = gen.crush512(n=2)
    finally:
        gen.set_bond_builder("cpu")
    for p in range(s_cpu.n_particles):
        sl = s_cpu.particle_slice(p)
        _same_up_to_boundary(s_gpu.particle_conn(p), s_cpu.particle_conn(p), s_cpu.pos[sl], 3 * s_cpu.meta["h"][p])


def _near_formula(pos, marked, r):
    """The reference's nonlocal boundary pass (exp_dict.py:1231-1248) as numpy evaluates it: q is
    kept when sqrt((dx*dx + dy*dy) + dz*dz) <= r for some marked node (itself included)."""
    near = np.zeros(len(pos), dtype=bool)
    for e in np.nonzero(marked)[0]:
        d = pos - pos[e]
        near |= np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]) <= r
    return near


def test_near_marked_nodes_equal_the_reference_test():
    """pd_query_near on jittered lattices with random marked nodes, plus points placed within a
    few ulps of the radius of a marked point: the same flags as the reference's test, bit for
    bit, with several particles in one call (an empty one among them)."""
    rng = np.random.default_rng(11)
    sets, marks, radii = [], [], []
    for kind, size, h in (("sphere", 1.0e-3, 1e-4), ("cube", 0.7e-3, 0.9e-4), ("ellipsoid", (1.1e-3, 0.6e-3, 0.8e-3), 1e-4)):
        P = gen.lattice(kind, size, h) + rng.uniform(-0.05 * h, 0.05 * h, size=(len(gen.lattice(kind, size, h)), 3))
        m = rng.random(len(P)) < 0.05
        sets.append(P)
        marks.append(m)
        radii.append(0.5 * h * 1.37)
    # a marked point and points at r * (1 + k eps) in random directions
    r = 1e-4
    c = np.array([[2e-3, -1e-3, 5e-4]])
    dirs = rng.normal(size=(400, 3))
    dirs /= np.linalg.norm(dirs, axis=1)[:, None]
    scale = r * (1.0 + rng.integers(-4, 5, size=400) * np.finfo(float).eps)
    pts = np.concatenate([c, c + dirs * scale[:, None]])
    m = np.zeros(len(pts), dtype=bool)
    m[0] = True
    sets += [pts, np.zeros((0, 3))]
    marks += [m, np.zeros(0, dtype=bool)]
    radii += [r, 1e-4]
    got = gen.near_gpu(sets, marks, radii)
    for P, m, rr, g in zip(sets, marks, radii, got):
        np.testing.assert_array_equal(g, _near_formula(P, m, rr))
    assert 0 < got[3].sum() < len(pts)  # both sides of the radius are exercised


def test_boundary_nodes_same_with_either_builder():
    rng = np.random.default_rng(5)
    h = 1e-4
    P = gen.lattice("sphere", 1.2e-3, h) + rng.uniform(-0.05 * h, 0.05 * h, size=(len(gen.lattice("sphere", 1.2e-3, h)), 3))
    conn = gen.bonds(P, 3 * h)
    cpu = gen.boundary_nodes(P, conn, 0.6 * h)
    gen.set_bond_builder("gpu")
    try:
        gpu = gen.boundary_nodes(P, conn, 0.6 * h)
    finally:
        gen.set_bond_builder("cpu")
    np.testing.assert_array_equal(cpu, gpu)
    assert 0 < len(cpu) < len(P)
