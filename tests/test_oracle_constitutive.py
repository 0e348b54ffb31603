"""Pins of the CPU oracle's constitutive math (CPU only).

The reference's util tests (rust/crates/util/src/tests.rs, run in f64 per
util/src/lib.rs:27-30) check every analytic derivative against central finite
differences on a fixed list of position gradients plus random ones with
|det F| in (0.1, 10) made positive, over the parameter sets of
util/src/elastic.rs:679-696.  The same checks are re-derived here against the
oracle's restatement, plus known answers worked out by hand.
"""

import math

import numpy as np
import pytest

import oracle

# util/src/elastic.rs:679-696
LAME = [(1e4, 0.3), (1e6, 0.3), (1e4, 0.0), (0.0, 0.4)]
INVISCID = [(100.0, 2), (1000.0, 2), (100.0, 7), (1000.0, 7)]


def fixed_gradients():
    """The hand-picked samples of util/src/tests.rs run_with_random_position_gradients."""
    rows = [
        [[1, 0, 0], [0, 1, 0], [0, 0, 1]],
        [[0, -1, 0], [1, 0, 0], [0, 0, 1]],
        [[0, 0, -1], [0, 1, 0], [1, 0, 0]],
        [[1, 0, 0], [0, 0, -1], [0, 1, 0]],
        [[3, 0, 0], [0, 2, 0], [0, 0, 1]],
        [[1, 0, 0], [0, 2, 0], [0, 0, 1]],
        [[0, -1, 0], [1, 0, 0], [0, 0, 2]],
        [[0, -1, 0], [2, 0, 0], [0, 0, 1]],
        [[0, -2, 0], [1, 0, 0], [0, 0, 1]],
    ]
    return [np.array(r, np.float64) for r in rows]


def random_gradients(n, seed=42):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        F = rng.random((3, 3))
        d = abs(np.linalg.det(F))
        if 1e-1 < d < 1e1:
            out.append(F if np.linalg.det(F) > 0 else -F)
    return out


def col_major(F):
    return np.asarray(F, np.float64).T.reshape(9)  # nalgebra storage


def from_col_major(a):
    return np.asarray(a, np.float64).reshape(3, 3).T


def fd_gradient(fun, F, h):
    G = np.zeros((3, 3))
    for r in range(3):
        for c in range(3):
            a, b = F.copy(), F.copy()
            a[r, c] += h
            b[r, c] -= h
            G[r, c] = (fun(a) - fun(b)) / (2 * h)
    return G


def check_gradient(energy, piola, F, h=1e-6, eps=1e-4):
    fd = fd_gradient(energy, F, h)
    an = piola(F)
    # util/src/tests.rs test_scalar_from_matrix: tiny entries compared absolutely
    for f, a in zip(fd.ravel(), an.ravel()):
        if abs(f) < 1e-2:
            assert abs(a) < 1e-2 + 1e-6 * np.abs(an).max()
        else:
            assert abs(f - a) / abs(f) < eps, (f, a)


def test_lame_parameters_known_values():
    # Wikipedia's Lamé formulas (util/src/elastic.rs:52-64)
    assert math.isclose(oracle.mu(1e4, 0.3), 1e4 / 2 / 1.3)
    assert math.isclose(oracle.lambda_(1e4, 0.3), 1e4 * 0.3 / 1.3 / 0.4)
    assert oracle.mu(0.0, 0.4) == 0.0


def test_kernel_quadratic_known_values_and_partition_of_unity():
    # cpu/src/kernels.rs:17-26
    assert oracle.kernel_quadratic(0.0) == 0.75
    assert oracle.kernel_quadratic(0.5) == 0.5
    assert oracle.kernel_quadratic(-1.0) == 0.125
    assert oracle.kernel_quadratic(1.5) == 0.0
    assert oracle.kernel_quadratic(2.0) == 0.0
    for x in np.linspace(0.5, 1.5, 41):
        s = sum(oracle.kernel_quadratic(x - i) for i in range(3))
        assert math.isclose(s, 1.0, rel_tol=1e-14)
        # first moment vanishes: the APIC affine terms conserve momentum
        m1 = sum(oracle.kernel_quadratic(x - i) * (i - x) for i in range(3))
        assert abs(m1) < 1e-14


@pytest.mark.parametrize("E,nu", LAME)
def test_neo_hookean_stress_is_energy_gradient(E, nu):
    mu, la = oracle.mu(E, nu), oracle.lambda_(E, nu)
    energy = lambda F: oracle.energy("neo_hookean", mu, la, col_major(F))
    piola = lambda F: from_col_major(oracle.piola("neo_hookean", mu, la, col_major(F)))
    for F in fixed_gradients() + random_gradients(50):
        if np.linalg.det(F) <= 0:
            continue
        scale = max(mu, la, 1.0)
        check_gradient(lambda G: energy(G) / scale, lambda G: piola(G) / scale, F)


@pytest.mark.parametrize("K,gamma", INVISCID)
def test_inviscid_stress_is_energy_gradient(K, gamma):
    energy = lambda F: oracle.energy("inviscid", K, gamma, col_major(F))
    piola = lambda F: from_col_major(oracle.piola("inviscid", K, gamma, col_major(F)))
    for F in fixed_gradients() + random_gradients(50, seed=7):
        if np.linalg.det(F) <= 0:
            continue
        check_gradient(lambda G: energy(G) / K, lambda G: piola(G) / K, F)


@pytest.mark.parametrize("E,nu", LAME)
def test_fixed_corotated_stress_is_energy_gradient(E, nu):
    # addition: psi = mu |F - R|^2 + lambda/2 (J - 1)^2
    mu, la = oracle.mu(E, nu), oracle.lambda_(E, nu)
    energy = lambda F: oracle.energy("fixed_corotated", mu, la, col_major(F))
    piola = lambda F: from_col_major(oracle.piola("fixed_corotated", mu, la, col_major(F)))
    for F in random_gradients(50, seed=9):
        s = np.linalg.svd(F, compute_uv=False)
        if min(abs(s[0] - s[1]), abs(s[1] - s[2])) < 1e-3:
            continue  # R is not differentiable where singular values meet
        scale = max(mu, la, 1.0)
        check_gradient(lambda G: energy(G) / scale, lambda G: piola(G) / scale, F)


def test_neo_hookean_known_answer():
    # diag(2, 1, 1): P = mu F + (lambda ln J - mu)/J cof F, cof = diag(1, 2, 2)
    mu, la = 10.0, 20.0
    F = np.diag([2.0, 1.0, 1.0])
    P = from_col_major(oracle.piola("neo_hookean", mu, la, col_major(F)))
    d3 = (la * math.log(2.0) - mu) / 2.0
    np.testing.assert_allclose(np.diag(P), [mu * 2 + d3 * 1, mu + d3 * 2, mu + d3 * 2], rtol=1e-14)
    e = oracle.energy("neo_hookean", mu, la, col_major(F))
    assert math.isclose(e, mu / 2 * (6 - 3) - mu * math.log(2) + la / 2 * math.log(2) ** 2, rel_tol=1e-14)
    assert oracle.energy("neo_hookean", mu, la, col_major(np.eye(3))) == 0.0


def test_viscosity_known_answer():
    # util/src/elastic.rs:670-677: 2 mu_d sym(C) + mu_b tr(C) I
    C = np.arange(9, dtype=np.float64).reshape(3, 3)
    S = from_col_major(oracle.cauchy_viscosity(0.5, 0.25, col_major(C)))
    np.testing.assert_allclose(S, 0.5 * (C + C.T) + 0.25 * np.trace(C) * np.eye(3), rtol=1e-14)


@pytest.mark.parametrize("F", random_gradients(30, seed=3) + fixed_gradients()
                         + [np.diag([1.0, 1.0, 0.0]), np.zeros((3, 3)), -np.eye(3)])
def test_svd_reconstructs_and_is_orthogonal(F):
    U, S, V = oracle.svd3(col_major(F))
    U, V = from_col_major(U), from_col_major(V)
    np.testing.assert_allclose(U @ np.diag(S) @ V.T, F, atol=1e-12)
    np.testing.assert_allclose(U.T @ U, np.eye(3), atol=1e-12)
    np.testing.assert_allclose(V.T @ V, np.eye(3), atol=1e-12)
    assert np.all(S >= 0) and np.all(np.diff(S) <= 1e-15)
    np.testing.assert_allclose(S, np.linalg.svd(F, compute_uv=False), atol=1e-12)


def sand_by_hand(s, mu, la, alpha):
    """advance_particles.rs:48-71 on singular values (diagonal F)."""
    e = np.log(s)
    e_tr = e.sum()
    e_hat = e - e_tr / 3
    n = np.linalg.norm(e_hat)
    if e_tr < 0 and n > 0:
        dg = n + (3 * la + 2 * mu) / 2 / mu * e_tr * alpha
        if dg > 0:
            return np.exp(e - dg / n * e_hat)
        return s
    return np.ones(3)


@pytest.mark.parametrize("s", [[0.9, 0.95, 1.0], [0.8, 1.0, 1.1], [1.05, 1.0, 0.99], [1.1, 1.2, 1.3], [0.7, 0.7, 0.7]])
def test_sand_return_map_known_answers(s):
    mu, la = oracle.mu(3.5e5, 0.3), oracle.lambda_(3.5e5, 0.3)
    alpha = oracle.friction_angle_to_alpha(math.radians(35.0))
    F = np.diag(s)
    out = from_col_major(oracle.project_sand(mu, la, alpha, col_major(F)))
    np.testing.assert_allclose(out, np.diag(sand_by_hand(np.array(s), mu, la, alpha)), atol=1e-13)


def test_sand_projection_commutes_with_rotation():
    rng = np.random.default_rng(1)
    mu, la, alpha = 1e4, 2e4, 0.3
    for _ in range(20):
        Q1, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        Q2, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        s = rng.uniform(0.7, 1.2, 3)
        F = Q1 @ np.diag(s) @ Q2.T
        out = from_col_major(oracle.project_sand(mu, la, alpha, col_major(F)))
        exp = Q1 @ np.diag(sand_by_hand(s, mu, la, alpha)) @ Q2.T
        np.testing.assert_allclose(out, exp, atol=1e-12)


def test_fluid_projection_keeps_volume_and_rotation():
    # advance_particles.rs:77-85: singular values -> geometric mean
    rng = np.random.default_rng(2)
    for _ in range(20):
        Q1, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        Q2, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        s = rng.uniform(0.5, 1.5, 3)
        F = Q1 @ np.diag(s) @ Q2.T
        out = from_col_major(oracle.project_fluid(col_major(F)))
        g = np.prod(s) ** (1 / 3)
        np.testing.assert_allclose(out, g * Q1 @ Q2.T, atol=1e-12)


def test_snow_projection_clamps_and_tracks_volume():
    # addition (Stomakhin et al. 2013)
    F = np.diag([0.9, 1.0, 1.02])
    out, jp = oracle.project_snow(2.5e-2, 7.5e-3, col_major(F), 1.0)
    np.testing.assert_allclose(from_col_major(out), np.diag([0.975, 1.0, 1.0075]), atol=1e-14)
    assert math.isclose(jp, (0.9 * 1.02) / (0.975 * 1.0075), rel_tol=1e-14)


def test_friction_angle_to_alpha():
    # addition: Klar et al. 2016
    s = math.sin(math.radians(35.0))
    assert math.isclose(oracle.friction_angle_to_alpha(math.radians(35.0)), math.sqrt(2 / 3) * 2 * s / (3 - s))
