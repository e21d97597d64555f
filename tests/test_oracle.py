"""Pin the CPU oracle against the reference PySPH's own outputs.

The golden fixtures were produced by the reference (``tests/golden/
make_golden.py``).  Given the reference's neighbour lists in the reference's
order, the oracle's pair sums must match bit for bit (FP64, no FMA); its own
neighbour search must give identical index sets; a full oracle step must
match the reference step to FP64 round-off.
"""
import numpy as np
import pytest

import oracle
from golden_util import csr_sets, inputs, load, normwise


def test_kernel_values_bit_exact():
    g = load("kernel")
    rs = g["r_over_h"]
    for dim in (1, 2, 3):
        for h in (0.1, 0.37, 1.0):
            d = np.array([0.6, -0.48, 0.64])[:dim]
            d = d / np.linalg.norm(d)
            for n, r in enumerate(rs):
                q = np.zeros(3)
                q[:dim] = d * r * h
                w = oracle.cubic_w(dim, (0, 0, 0), tuple(q), h)
                gr = oracle.cubic_grad(dim, (0, 0, 0), tuple(q), h)
                assert w == g["w_d%d_h%g" % (dim, h)][n]
                np.testing.assert_array_equal(gr, g["g_d%d_h%g" % (dim, h)][n])


def test_square4_functions():
    g = load("square4")
    props = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    off, idx = oracle.neighbors(props, props, cell_size=2.0, same=True)
    for kind, nout, params in (("rho", 1, {}), ("pgrad", 2, {}),
                               ("avisc", 3, {"alpha": 1.0, "beta": 1.0}),
                               ("xsph", 2, {"eps": 0.5})):
        res = oracle.pair_sum(kind, props, props, off, idx, 2, params, nout)
        for k in range(nout):
            np.testing.assert_allclose(res[k], g["%s_%d" % (kind, k)], rtol=1e-14, atol=1e-14)


def _check_neighbours(g, dest, src, props_d, props_s, cell_size):
    off, idx = oracle.neighbors(props_d, props_s, cell_size, same=(dest == src))
    ro = g["nbr_%s_%s_offsets" % (dest, src)]
    ri = g["nbr_%s_%s_index" % (dest, src)]
    assert csr_sets(off, idx) == csr_sets(ro, ri)
    if dest == src:
        last = idx[off[1:] - 1]
        np.testing.assert_array_equal(last, np.arange(len(off) - 1))
        np.testing.assert_array_equal(ri[ro[1:] - 1], np.arange(len(ro) - 1))


@pytest.mark.parametrize("name,dim", [("drop_step", 2), ("cube_step", 3)])
def test_neighbour_sets_match_reference(name, dim):
    g = load(name)
    p = inputs(g, "fluid")
    _check_neighbours(g, "fluid", "fluid", p, p, 2.0 * p["h"].max())


def test_dam_neighbour_sets_match_reference():
    g = load("dam_step")
    f, w = inputs(g, "fluid"), inputs(g, "boundary")
    cs = 2.0 * max(f["h"].max(), w["h"].max())
    _check_neighbours(g, "fluid", "fluid", f, f, cs)
    _check_neighbours(g, "fluid", "boundary", f, w, cs)


def test_drop_pair_sums_bit_exact_with_reference_lists():
    """Same neighbour order as the reference -> identical FP64 sums."""
    g = load("drop_step")
    p = inputs(g, "fluid")
    off = g["nbr_fluid_fluid_offsets"]
    idx = g["nbr_fluid_fluid_index"]
    rho = oracle.pair_sum("rho", p, p, off, idx, 2)[0]
    np.testing.assert_array_equal(rho, g["eval1_fluid_rho"])
    p2 = dict(p, rho=g["eval1_fluid_rho"], p=g["eval1_fluid_p"], cs=g["eval1_fluid_cs"])
    pt, ct = oracle.tait(dict(p, rho=g["eval1_fluid_rho"]), 1400.0, 1.0)
    np.testing.assert_array_equal(pt, g["eval1_fluid_p"])
    np.testing.assert_array_equal(ct, g["eval1_fluid_cs"])
    pg = oracle.pair_sum("pgrad", p2, p2, off, idx, 2, nout=2)
    np.testing.assert_array_equal(pg[0], g["eval1_k_pgrad_fluid_u"])
    np.testing.assert_array_equal(pg[1], g["eval1_k_pgrad_fluid_v"])
    av = oracle.pair_sum("avisc", p2, p2, off, idx, 2, {"alpha": 0.01, "beta": 0.0}, 3)
    for k, c in enumerate("uvw"):
        np.testing.assert_array_equal(av[k], g["eval1_k_avisc_fluid_" + c])
    xs = oracle.pair_sum("xsph", p2, p2, off, idx, 2, {"eps": 0.5}, 2)
    np.testing.assert_array_equal(xs[0], g["eval1_k_xsph_fluid_x"])
    np.testing.assert_array_equal(xs[1], g["eval1_k_xsph_fluid_y"])


def _step_problem(g, arrays, ops, dim, scheme):
    prob = oracle.Problem(arrays, ops, dim)
    getattr(prob, "integrate_" + scheme)(float(g["dt"]))
    return prob


def _cmp_step(g, prob, names, tol):
    for arr in names:
        for p_ in ("x", "y", "z", "u", "v", "w", "rho", "p", "cs"):
            key = "out_%s_%s" % (arr, p_)
            if key in g:
                err = normwise(prob.arrays[arr][p_], g[key])
                assert err <= tol, (key, err)


def test_drop_euler_step_matches_reference():
    g = load("drop_step")
    prob = _step_problem(g, {"fluid": inputs(g, "fluid")}, oracle.drop_ops(), 2, "euler")
    _cmp_step(g, prob, ["fluid"], 1e-13)
    for c in "uvw":
        assert normwise(prob.k[("k1", 3)][" uvw".index(c) - 1], g["eval1_k_avisc_fluid_" + c]) < 1e-13


def test_drop_ten_euler_steps_match_reference():
    g = load("drop_traj10")
    prob = oracle.Problem({"fluid": inputs(g, "fluid")}, oracle.drop_ops(), 2)
    for _ in range(int(g["steps"])):
        prob.integrate_euler(float(g["dt"]))
    for p_ in ("x", "y", "u", "v", "rho", "p", "cs"):
        assert normwise(prob.arrays["fluid"][p_], g["final_" + p_]) < 1e-11, p_


def test_dam_rk2_step_matches_reference():
    g = load("dam_step")
    arrays = {"fluid": inputs(g, "fluid"), "boundary": inputs(g, "boundary")}
    prob = _step_problem(g, arrays, oracle.dam_ops(float(g["dx"]), float(g["c0"])), 2, "rk2")
    _cmp_step(g, prob, ["fluid", "boundary"], 1e-13)
    kb = prob.k[("k2", 4)]
    assert normwise(kb[0], g["eval2_k_bforce_fluid_u"]) < 1e-13
    assert normwise(kb[1], g["eval2_k_bforce_fluid_v"]) < 1e-13


def test_cube_rk2_step_matches_reference():
    g = load("cube_step")
    prob = _step_problem(g, {"fluid": inputs(g, "fluid")}, oracle.cube_ops(), 3, "rk2")
    _cmp_step(g, prob, ["fluid"], 1e-13)
    for c, k in zip("uvw", range(3)):
        assert normwise(prob.k[("k2", 2)][k], g["eval2_k_pgrad_fluid_" + c]) < 1e-13


def test_square4_momentum_and_density_rate():
    """MomentumEquation (eta stored) and SPHDensityRate on the square."""
    g = load("square4_momentum")
    props = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    off, idx = oracle.neighbors(props, props, cell_size=2.0, same=True)
    res = oracle.pair_sum("momentum", props, props, off, idx, 2,
                          {"alpha": 1.0, "beta": 1.0, "eta": 0.1}, 3)
    for k in range(3):
        np.testing.assert_allclose(res[k], g["momentum_%d" % k], rtol=1e-14, atol=1e-14)
    dr = oracle.pair_sum("drho", props, props, off, idx, 2)[0]
    np.testing.assert_allclose(dr, g["drho_0"], rtol=1e-14, atol=1e-14)


def test_fluid_solver_pair_sums_bit_exact_with_reference_lists():
    g = load("fluid_step")
    p = inputs(g, "fluid")
    off = g["nbr_fluid_fluid_offsets"]
    idx = g["nbr_fluid_fluid_index"]
    pt, ct = oracle.tait(p, 100.0, 1.0)
    p2 = dict(p, p=pt, cs=ct)
    dr = oracle.pair_sum("drho", p2, p2, off, idx, 2)[0]
    np.testing.assert_array_equal(dr, g["eval1_k_density_fluid_rho"])
    mo = oracle.pair_sum("momentum", p2, p2, off, idx, 2,
                         {"alpha": 0.01, "beta": 0.0, "eta": 0.1}, 3)
    for k, c in enumerate("uvw"):
        np.testing.assert_array_equal(mo[k], g["eval1_k_mom_fluid_" + c])


def test_fluid_solver_rk2_step_matches_reference():
    g = load("fluid_step")
    prob = _step_problem(g, {"fluid": inputs(g, "fluid")}, oracle.fluid_ops(), 2, "rk2")
    _cmp_step(g, prob, ["fluid"], 1e-13)


# -- the other integrators of solver/integrator.py:650-912 -------------------

def _multi_step(g, arrays, ops, dim, scheme, tol_step, tol_final):
    prob = _step_problem(g, arrays, ops, dim, scheme)
    _cmp_step(g, prob, list(arrays), tol_step)
    if "steps" in g:
        for _ in range(int(g["steps"]) - 1):
            getattr(prob, "integrate_" + scheme)(float(g["dt"]))
        for p_ in ("x", "y", "u", "v", "rho", "p", "cs"):
            assert normwise(prob.arrays["fluid"][p_], g["final_" + p_]) < tol_final, p_
    return prob


@pytest.mark.parametrize("scheme", ["rk4", "pc"])
def test_drop_step_matches_reference(scheme):
    g = load("drop_" + scheme)
    assert int(g["n_evals"]) == {"rk4": 4, "pc": 2}[scheme]
    _multi_step(g, {"fluid": inputs(g, "fluid")}, oracle.drop_ops(), 2, scheme, 1e-13, 1e-12)
    if scheme == "rk4":
        prob = _step_problem(g, {"fluid": inputs(g, "fluid")}, oracle.drop_ops(), 2, scheme)
        for c, k in zip("uv", range(2)):
            assert normwise(prob.k[("k3", 2)][k], g["eval3_k_pgrad_fluid_" + c]) < 1e-13


@pytest.mark.parametrize("scheme", ["rk4", "pc"])
def test_fluid_solver_step_matches_reference(scheme):
    g = load("fluid_" + scheme)
    _multi_step(g, {"fluid": inputs(g, "fluid")}, oracle.fluid_ops(), 2, scheme, 1e-13, 1e-12)


def test_cube_leapfrog_step_matches_reference():
    g = load("cube_leapfrog")
    assert int(g["n_evals"]) == 3
    prob = _step_problem(g, {"fluid": inputs(g, "fluid")}, oracle.cube_ops(), 3, "leapfrog")
    _cmp_step(g, prob, ["fluid"], 1e-13)
    # the position calc was evaluated once, on the predicted velocities
    for c in "xyz":
        assert normwise(prob.k[("k1", 4)]["xyz".index(c)], g["eval2_k_step_fluid_" + c]) < 1e-13


def test_leapfrog_2d_position_correction_index_error():
    """2D velocity calcs with three outputs (Monaghan AV) index past the two
    position updates in add_correction_for_position (integrator.py:861-865);
    the reference raises IndexError there and so does the oracle."""
    g = load("drop_step")
    prob = oracle.Problem({"fluid": inputs(g, "fluid")}, oracle.drop_ops(), 2)
    with pytest.raises(IndexError):
        prob.integrate_leapfrog(1e-5)


def test_variable_h_neighbour_sets_match_reference():
    """Particles(variable_h=True): the symmetric union of VarHNbrParticleLocator
    (base/nnps.pyx:654-749), a strict superset of the fixed-h sets here."""
    g = load("drop_varh")
    p = inputs(g, "fluid")
    off, idx = oracle.neighbors(p, p, 2 * p["h"].max(), 2.0, same=True, variable_h=True)
    ref = csr_sets(g["nbr_fluid_fluid_offsets"], g["nbr_fluid_fluid_index"])
    assert csr_sets(off, idx) == ref
    o2, i2 = oracle.neighbors(p, p, 2 * p["h"].max(), 2.0, same=True)
    assert o2[-1] < off[-1]
    # symmetric: j in N(i) <=> i in N(j)
    pairs = {(i, j) for i, s in enumerate(ref) for j in s}
    assert all((j, i) in pairs for (i, j) in pairs)


def test_variable_h_euler_step_matches_reference():
    g = load("drop_varh")
    prob = oracle.Problem({"fluid": inputs(g, "fluid")}, oracle.drop_ops(), 2, variable_h=True)
    prob.integrate_euler(float(g["dt"]))
    _cmp_step(g, prob, ["fluid"], 1e-13)


def _periodic_case():
    g = load("periodic")
    n = int(g["n_real"])
    p = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    return g, n, p


def test_periodic_neighbour_sets_match_reference():
    """PeriodicDomain along x: the reference's lists over real particles and
    the ghost copies it appends (cell.pyx:1277-1376), ghosts mapped to the
    particle they copy, equal the oracle's lists over periodic images."""
    g, n, p = _periodic_case()
    origin = g["ghost_origin"]
    ref = csr_sets(g["nbr_offsets"], g["nbr_index"])
    ref = [{(j if j < n else int(origin[j - n])) for j in s} for s in ref]
    prob = oracle.Problem({"fluid": p}, [], 2, periodic=(float(g["xmin"]), float(g["xmax"])))
    off, idx = prob.neighbours("fluid", "fluid")
    _, gor = prob._source("fluid")
    got = [{(j if j < n else int(gor[j - n])) for j in s} for s in csr_sets(off, idx)]
    assert got == ref
    # the boundary rows see images: particle 0 has as many neighbours as an interior one
    assert len(ref[0]) == len(ref[5])


def test_periodic_pair_sums_bit_exact_with_reference_lists():
    """Given the reference's lists and ghost positions, every pair function
    sums to the same FP64 bits (ghosts carrying their originals' state)."""
    g, n, p = _periodic_case()
    origin, shift = g["ghost_origin"], g["ghost_shift"]
    ext = {k: np.concatenate([v, v[origin]]) for k, v in p.items()}
    ext["x"] = np.concatenate([p["x"], p["x"][origin] + shift])
    off, idx = g["nbr_offsets"], g["nbr_index"]
    for name, params, nout in (("pgrad", {}, 2), ("avisc", {"alpha": 1.0, "beta": 1.0}, 3),
                               ("xsph", {"eps": 0.5}, 2), ("rho", {}, 1)):
        res = oracle.pair_sum(name, p, ext, off, idx, 2, params, nout)
        for k in range(nout):
            np.testing.assert_array_equal(res[k], g["%s_%d" % (name, k)])


def test_periodic_images_are_the_minimum_images():
    """With particles past the end of the period (x is never wrapped), the
    oracle's lists are exactly the sources within radius among every
    particle's images x_j + {-L, 0, L} (brute force)."""
    from pysph_gb300 import workloads as W
    props = W.periodic_strip(vel_std=1.0)
    props["x"] = props["x"] + 0.07
    prob = oracle.Problem({"fluid": props}, [], 2, periodic=(0.0, 1.0))
    off, idx = prob.neighbours("fluid", "fluid")
    _, gor = prob._source("fluid")
    n = len(props["x"])
    x, y, h = props["x"], props["y"], props["h"]
    for i in range(n):
        got = sorted(int(j) if j < n else int(gor[j - n]) for j in idx[off[i]:off[i + 1]])
        ref = sorted(j for j in range(n) for s in (-1.0, 0.0, 1.0)
                     if ((x[j] + s if s else x[j]) - x[i]) ** 2 + (y[j] - y[i]) ** 2 < (2 * h[i]) ** 2)
        assert got == ref, i


def test_adke_functions_match_reference():
    """ADKE (adke_funcs.pyx) on the jittered-h drop, variable-h lists: the
    reference's neighbour sets before and after the smoothing update, the
    pilot density and the divergence over the reference's lists bit for bit,
    the smoothing update and the conduction coefficient to FP64 round-off."""
    g = load("adke")
    props = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    cell = 2.0 * props["h"].max()
    off, idx = oracle.neighbors(props, props, cell, same=True, variable_h=True)
    assert csr_sets(off, idx) == csr_sets(g["nbr0_offsets"], g["nbr0_index"])
    h0 = float(g["h0"])
    rhop = oracle.pair_sum("pilotrho", props, props, g["nbr0_offsets"], g["nbr0_index"], 2,
                           {"h0": h0}, nout=1)[0]
    np.testing.assert_array_equal(rhop, g["rhop"])
    st = dict(props, rhop=g["rhop"])
    h = oracle.adke_smoothing(st, h0, float(g["k"]), float(g["eps"]))
    np.testing.assert_allclose(h, g["h_new"], rtol=1e-15, atol=0)
    st["h"] = g["h_new"]
    off1, idx1 = oracle.neighbors(st, st, 2.0 * st["h"].max(), same=True, variable_h=True)
    assert csr_sets(off1, idx1) == csr_sets(g["nbr1_offsets"], g["nbr1_index"])
    div = oracle.pair_sum("vdiv", st, st, g["nbr1_offsets"], g["nbr1_index"], 2, nout=1)[0]
    np.testing.assert_array_equal(div, g["div"])
    assert not g["div_1"].any() and not g["div_2"].any()
    st["div"] = g["div"]
    q = oracle.adke_conduction(st, float(g["g1"]), float(g["g2"]))
    np.testing.assert_array_equal(q, g["q"])
