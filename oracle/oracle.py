"""ctypes binding of oracle/_build/libsv_oracle.so (TEST INFRASTRUCTURE ONLY).

The library restates rust/crates/cpu (the reference MPM substep) and
rust/crates/util/src/elastic.rs in C++; see sv_oracle.h for what is pinned
and how.
"""

from __future__ import annotations

import ctypes as ct
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libsv_oracle.so"

u32p = ct.POINTER(ct.c_uint32)
i32p = ct.POINTER(ct.c_int32)
f32p = ct.POINTER(ct.c_float)
f64p = ct.POINTER(ct.c_double)


class OParticles(ct.Structure):
    _fields_ = [
        ("n", ct.c_uint64),
        ("flags", u32p),
        ("positions", f32p),
        ("position_gradients", f32p),
        ("velocities", f32p),
        ("velocity_gradients", f32p),
        ("elastic_energies", f32p),
        ("collider_bits", u32p),
        ("mass", f32p),
        ("initial_volume", f32p),
        ("viscosity_dynamic", f32p),
        ("viscosity_bulk", f32p),
        ("mu", f32p),
        ("lambda_", f32p),
        ("sand_alpha", f32p),
        ("exponent", i32p),
        ("bulk_modulus", f32p),
        ("model", u32p),
        ("hardening", f32p),
        ("crit_compression", f32p),
        ("crit_stretch", f32p),
        ("plastic_j", f32p),
    ]


class OConsts(ct.Structure):
    _fields_ = [
        ("grid_node_size", ct.c_float),
        ("domain_min", ct.c_float * 3),
        ("domain_max", ct.c_float * 3),
        ("ground_mode", ct.c_int32),
        ("ground_axis", ct.c_int32),
        ("ground_height", ct.c_float),
    ]


class OFrameInput(ct.Structure):
    """svo_frame_input (sv_oracle.h)."""

    _fields_ = [
        ("frames_per_second", ct.c_uint32),
        ("frame", ct.c_uint32),
        ("has_b", ct.c_uint32),
        ("gravity_a", ct.c_float * 3),
        ("gravity_b", ct.c_float * 3),
        ("goal_flags_a", u32p),
        ("goal_flags_b", u32p),
        ("goal_positions_a", f32p),
        ("goal_positions_b", f32p),
        ("n_vertices", ct.c_uint32),
        ("n_triangles", ct.c_uint32),
        ("triangles", u32p),
        ("triangle_collider", u32p),
        ("vertex_positions_a", f32p),
        ("vertex_positions_b", f32p),
        ("friction_a", f32p),
        ("friction_b", f32p),
        ("damping_a", f32p),
        ("damping_b", f32p),
        ("leaf_size", ct.c_float),
    ]


def build() -> Path:
    """Builds the oracle with its Makefile (g++ only)."""
    r = subprocess.run(["make", "-C", str(HERE), "-s"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


_lib = None


def lib() -> ct.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = ct.CDLL(str(LIB))
        d = ct.c_double
        sig = {
            "svo_mu": (d, [d, d]),
            "svo_lambda": (d, [d, d]),
            "svo_kernel_quadratic": (d, [d]),
            "svo_energy_neo_hookean": (d, [d, d, f64p]),
            "svo_piola_neo_hookean": (None, [d, d, f64p, f64p]),
            "svo_energy_inviscid": (d, [d, ct.c_int32, f64p]),
            "svo_piola_inviscid": (None, [d, ct.c_int32, f64p, f64p]),
            "svo_energy_fixed_corotated": (d, [d, d, f64p]),
            "svo_piola_fixed_corotated": (None, [d, d, f64p, f64p]),
            "svo_cauchy_viscosity": (None, [d, d, f64p, f64p]),
            "svo_svd3": (None, [f64p, f64p, f64p, f64p]),
            "svo_project_sand": (ct.c_int, [d, d, d, f64p]),
            "svo_deterministic_grid_mass": (ct.c_uint64, [f32p, f32p, u32p, ct.c_uint64, ct.c_float, i32p, f32p,
                                                          ct.c_uint64]),
            "svo_project_fluid": (None, [f64p]),
            "svo_project_snow": (None, [d, d, f64p, f64p]),
            "svo_friction_angle_to_alpha": (d, [d]),
            "svo_create": (ct.c_void_p, [ct.POINTER(OParticles), ct.POINTER(OConsts), ct.c_int, ct.c_int]),
            "svo_destroy": (None, [ct.c_void_p]),
            "svo_step": (ct.c_int, [ct.c_void_p, ct.c_uint32, ct.c_float, f32p]),
            "svo_step_adaptive": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_double), ct.c_double, ct.c_float, f32p,
                                             u32p, f32p]),
            "svo_set_frame_input": (ct.c_int, [ct.c_void_p, ct.POINTER(OFrameInput)]),
            "svo_set_time": (None, [ct.c_void_p, ct.c_double]),
            "svo_get_time": (ct.c_double, [ct.c_void_p]),
            "svo_download": (None, [ct.c_void_p, ct.POINTER(OParticles)]),
            "svo_grid": (ct.c_uint64, [ct.c_void_p, i32p, f32p, f32p, ct.c_uint64]),
            "svo_p2g_only": (None, [ct.c_void_p, ct.c_float, f32p]),
            "svo_binning_keys": (None, [ct.c_uint64, f32p, u32p, ct.c_float, i32p, i32p, u32p]),
            "svo_stable_sort_perm": (None, [ct.c_uint64, u32p, u32p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a, t):
    return ct.cast(None, t) if a is None else a.ctypes.data_as(t)


def _m9(F):
    return np.ascontiguousarray(np.asarray(F, np.float64).reshape(9))


# ---- scalar constitutive functions (double precision)
def mu(E, nu):
    return lib().svo_mu(E, nu)


def lambda_(E, nu):
    return lib().svo_lambda(E, nu)


def kernel_quadratic(x):
    return lib().svo_kernel_quadratic(x)


def energy(model, a, b, F):
    F = _m9(F)
    L = lib()
    if model == "neo_hookean":
        return L.svo_energy_neo_hookean(a, b, _p(F, f64p))
    if model == "inviscid":
        return L.svo_energy_inviscid(a, int(b), _p(F, f64p))
    if model == "fixed_corotated":
        return L.svo_energy_fixed_corotated(a, b, _p(F, f64p))
    raise ValueError(model)


def piola(model, a, b, F):
    F = _m9(F)
    P = np.zeros(9)
    L = lib()
    if model == "neo_hookean":
        L.svo_piola_neo_hookean(a, b, _p(F, f64p), _p(P, f64p))
    elif model == "inviscid":
        L.svo_piola_inviscid(a, int(b), _p(F, f64p), _p(P, f64p))
    elif model == "fixed_corotated":
        L.svo_piola_fixed_corotated(a, b, _p(F, f64p), _p(P, f64p))
    else:
        raise ValueError(model)
    return P


def cauchy_viscosity(dyn, bulk, C):
    C = _m9(C)
    S = np.zeros(9)
    lib().svo_cauchy_viscosity(dyn, bulk, _p(C, f64p), _p(S, f64p))
    return S


def svd3(F):
    F = _m9(F)
    U, S, V = np.zeros(9), np.zeros(3), np.zeros(9)
    lib().svo_svd3(_p(F, f64p), _p(U, f64p), _p(S, f64p), _p(V, f64p))
    return U, S, V


def project_sand(mu_, lambda__, alpha, F):
    """Sand return map of F (advance_particles.rs:48-71).  Raises ValueError
    on the compressive branch with mu <= 0, where the reference asserts."""
    F = _m9(F).copy()
    if lib().svo_project_sand(mu_, lambda__, alpha, _p(F, f64p)) != 0:
        raise ValueError("sand return map: mu <= 0 under compression (the reference asserts mu > 0)")
    return F


def deterministic_grid_mass(positions, mass, flags, dx):
    """Node ids [m, 3] and fp32 masses of the reference's P2G mass summed in
    the canonical order (see svo_deterministic_grid_mass)."""
    x = np.ascontiguousarray(positions, np.float32)
    ms = np.ascontiguousarray(mass, np.float32)
    fl = np.ascontiguousarray(flags, np.uint32)
    n = len(ms)
    m = lib().svo_deterministic_grid_mass(_p(x, f32p), _p(ms, f32p), _p(fl, u32p), n, float(dx), None, None, 0)
    ids = np.zeros((m, 3), np.int32)
    out = np.zeros(m, np.float32)
    lib().svo_deterministic_grid_mass(_p(x, f32p), _p(ms, f32p), _p(fl, u32p), n, float(dx), _p(ids, i32p),
                                      _p(out, f32p), m)
    return ids, out


def project_fluid(F):
    F = _m9(F).copy()
    lib().svo_project_fluid(_p(F, f64p))
    return F


def project_snow(theta_c, theta_s, F, plastic_j):
    F = _m9(F).copy()
    j = np.array([plastic_j], np.float64)
    lib().svo_project_snow(theta_c, theta_s, _p(F, f64p), _p(j, f64p))
    return F, float(j[0])


def friction_angle_to_alpha(phi):
    return lib().svo_friction_angle_to_alpha(phi)


def binning_keys(positions, flags, dx, origin, nblocks):
    positions = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    n = positions.shape[0]
    flags = None if flags is None else np.ascontiguousarray(flags, np.uint32)
    o = np.ascontiguousarray(origin, np.int32)
    nb = np.ascontiguousarray(nblocks, np.int32)
    keys = np.zeros(n, np.uint32)
    lib().svo_binning_keys(n, _p(positions, f32p), _p(flags, u32p), float(dx), _p(o, i32p), _p(nb, i32p),
                           _p(keys, u32p))
    return keys


def stable_sort_perm(keys):
    keys = np.ascontiguousarray(keys, np.uint32)
    perm = np.zeros(keys.shape[0], np.uint32)
    lib().svo_stable_sort_perm(keys.shape[0], _p(keys, u32p), _p(perm, u32p))
    return perm


# ---- whole-state oracle
_FIELDS = [f[0] for f in OParticles._fields_ if f[0] != "n"]


class OracleState:
    """The reference substep restated on the CPU (fp32, or fp64 twin)."""

    def __init__(self, particles, consts, extras=None, fp64=False, threads=0):
        self._keep = particles.copy()
        s = self._struct(self._keep)
        c = OConsts()
        c.grid_node_size = consts.scaled_grid_node_size()
        for a in range(3):
            c.domain_min[a] = consts.scaled_domain_min()[a]
            c.domain_max[a] = consts.scaled_domain_max()[a]
        if extras is not None:
            c.ground_mode = extras.ground_mode
            c.ground_axis = extras.ground_axis
            c.ground_height = extras.ground_height
        self._h = lib().svo_create(ct.byref(s), ct.byref(c), 1 if fp64 else 0, int(threads))
        self.n = particles.n

    @staticmethod
    def _struct(p):
        s = OParticles()
        s.n = p.n
        for name in _FIELDS:
            arr = getattr(p, name, None)
            typ = dict(OParticles._fields_)[name]
            setattr(s, name, _p(arr, typ))
        return s

    def set_frame_input(self, frame):
        """frame: squishy_volumes_gb300.state.FrameData (its arrays are copied)."""
        s, keep = frame.to_struct(OFrameInput)
        rc = lib().svo_set_frame_input(self._h, ct.byref(s))
        if rc != 0:
            raise ValueError("invalid frame input")

    @property
    def time(self):
        return float(lib().svo_get_time(self._h))

    @time.setter
    def time(self, t):
        lib().svo_set_time(self._h, float(t))

    def step(self, n, dt, gravity):
        g = np.asarray(gravity, np.float32)
        return lib().svo_step(self._h, int(n), float(dt), _p(g, f32p))

    def step_adaptive(self, time, target, max_dt, gravity):
        """Adaptive substeps until target; returns (rc, substeps, time, limits)
        with limits = (dt_force, dt_scatter, dt_advance, velocity,
        deformation, sound, isolated, allowed)."""
        g = np.asarray(gravity, np.float32)
        t = ct.c_double(time)
        n = ct.c_uint32(0)
        lim = np.zeros(8, np.float32)
        rc = lib().svo_step_adaptive(self._h, ct.byref(t), float(target), float(max_dt), _p(g, f32p), ct.byref(n),
                                     _p(lim, f32p))
        return rc, int(n.value), float(t.value), lim

    def p2g_only(self, dt, gravity):
        g = np.asarray(gravity, np.float32)
        lib().svo_p2g_only(self._h, float(dt), _p(g, f32p))

    def download(self):
        out = self._keep.copy()
        if out.plastic_j is None:
            out.plastic_j = np.ones(out.n, np.float32)
        if out.elastic_energies is None:
            out.elastic_energies = np.zeros(out.n, np.float32)
        s = self._struct(out)
        lib().svo_download(self._h, ct.byref(s))
        return out

    def grid(self):
        m = lib().svo_grid(self._h, None, None, None, 0)
        ids = np.zeros((m, 3), np.int32)
        ms = np.zeros(m, np.float32)
        vs = np.zeros((m, 3), np.float32)
        lib().svo_grid(self._h, _p(ids, i32p), _p(ms, f32p), _p(vs, f32p), m)
        return ids, ms, vs

    def close(self):
        if self._h:
            lib().svo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
