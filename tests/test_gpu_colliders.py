"""Frame input and colliders through the C ABI against the fp32 oracle:
gravity interpolated inside the frame, particle goals, the reference's
Collide against triangle-mesh colliders with the (node, collider bits) grid
variants, frame boundaries, and adaptive steps with a collider."""

import numpy as np
import pytest

from squishy_volumes_gb300 import CudaState, Extras, FrameData, IoState
from squishy_volumes_gb300._abi import SV_HAS_GOAL, SV_TOMBSTONED, SvError
from squishy_volumes_gb300.scenes import Material, build_particles, jittered_box
from squishy_volumes_gb300.state import InputConsts

from test_gpu_parity import compare_states

pytestmark = pytest.mark.gpu

TOL = {"positions": 1e-5, "velocities": 1e-3, "position_gradients": 1e-4}
FPS = 24


def _consts(dx=0.05):
    return InputConsts(grid_node_size=dx, domain_min=(0.0, 0.0, 0.0), domain_max=(2.0, 2.0, 2.0))


def _falling_box(speed=-2.0, dims=(6, 6, 6), z0=0.52, dx=0.05, seed=1, E=1e4):
    rng = np.random.default_rng(seed)
    mat = Material("neo_hookean", youngs_modulus=E, poissons_ratio=0.3)
    return build_particles([(jittered_box(rng, (0.5, 0.5, z0), dims, dx / 2), mat, (0.0, 0.0, speed), dx / 2)])


def _quad(z, collider=0, x0=0.0, x1=2.0, y0=0.0, y1=2.0, flip=False):
    V = np.array([[x0, y0, z], [x1, y0, z], [x1, y1, z], [x0, y1, z]], np.float32)
    T = np.array([[0, 2, 1], [0, 3, 2]] if flip else [[0, 1, 2], [0, 2, 3]], np.uint32)
    return V, T, np.full(2, collider, np.uint32)


def _frame(frame=0, V=None, T=None, col=None, Vb=None, g_a=(0, 0, -9.8), g_b=(0, 0, -9.8), friction=0.5, damping=0.2,
           **goals):
    fd = FrameData(frames_per_second=FPS, frame=frame, gravity_a=g_a, gravity_b=g_b, leaf_size=0.25, **goals)
    if T is not None:
        nt = len(T)
        fd.triangles, fd.triangle_collider = T, col
        fd.vertex_positions_a, fd.vertex_positions_b = V, (V if Vb is None else Vb)
        fd.friction_a = fd.friction_b = np.full(nt, friction, np.float32)
        fd.damping_a = fd.damping_b = np.full(nt, damping, np.float32)
    return fd


def _pair(p, consts, fd, form=0, time=0.0):
    gpu = CudaState.from_io_state(IoState(time, p), consts, Extras(position_form=form))
    gpu.set_frame_input(fd)
    ref = __import__("oracle.oracle", fromlist=["OracleState"]).OracleState(p, consts, None, fp64=False)
    ref.set_frame_input(fd)
    ref.time = time
    return gpu, ref


def _check(gpu, ref, consts, bits=True):
    out, exp = gpu.download(), ref.download()
    np.testing.assert_array_equal(out.flags, exp.flags)
    if bits:
        np.testing.assert_array_equal(out.collider_bits, exp.collider_bits)
    live = (exp.flags & SV_TOMBSTONED) == 0
    compare_states(out, exp, live, tol=TOL, dx=consts.grid_node_size)
    return out, exp


def test_gravity_interpolated_inside_the_frame(cuda_lib, oracle_mod):
    p = _falling_box(speed=0.0)
    consts = _consts()
    fd = _frame(g_a=(0.0, 0.0, -9.8), g_b=(3.0, 0.0, 6.0))
    gpu, ref = _pair(p, consts, fd)
    n, dt = 300, 1e-4
    assert gpu.step(n, dt, (0, 0, 0)) == (0, n)
    assert ref.step(n, dt, (0, 0, 0)) == 0
    assert abs(gpu.time - ref.time) < 1e-12
    out, _ = _check(gpu, ref, consts)
    # the mean velocity is the time integral of the interpolated gravity
    t = np.arange(n) * dt * FPS
    g = (1 - t)[:, None] * np.array([0, 0, -9.8]) + t[:, None] * np.array([3.0, 0, 6.0])
    np.testing.assert_allclose(out.velocities.mean(0), (g * dt).sum(0), rtol=2e-3, atol=1e-4)
    gpu.close()


def test_goals_take_over_gravity(cuda_lib, oracle_mod):
    p = _falling_box(speed=0.0)
    consts = _consts()
    n = p.n
    flags = np.zeros(n, np.uint32)
    flags[: n // 2] = SV_HAS_GOAL
    goal = p.positions + np.array([0.05, 0.0, 0.0], np.float32)
    fd = _frame(goal_flags_a=flags, goal_flags_b=flags, goal_positions_a=goal, goal_positions_b=goal + 0.01)
    gpu, ref = _pair(p, consts, fd)
    assert gpu.step(50, 1e-4, (0, 0, 0)) == (0, 50)
    assert ref.step(50, 1e-4, (0, 0, 0)) == 0
    _check(gpu, ref, consts)
    gpu.close()


@pytest.mark.parametrize("form", [0, 1])
def test_box_lands_on_a_collider_quad(cuda_lib, oracle_mod, form):
    p = _falling_box()
    consts = _consts()
    V, T, col = _quad(0.45)
    gpu, ref = _pair(p, consts, _frame(V=V, T=T, col=col), form=form)
    n, dt = 400, 1e-4
    assert gpu.step(n, dt, (0, 0, 0)) == (0, n)
    assert ref.step(n, dt, (0, 0, 0)) == 0
    out, exp = _check(gpu, ref, consts)
    assert (out.collider_bits == 0x10001).sum() > 20  # the bottom layer is near the quad, above it
    assert out.positions[:, 2].min() > 0.45  # nothing went through
    gpu.close()


def test_thin_wall_keeps_two_bodies_apart(cuda_lib, oracle_mod):
    """Two bodies approach a wall (two colliders: its two faces) from both
    sides: particles on either side get different bits, their grid variants
    stay apart, and no particle crosses."""
    rng = np.random.default_rng(4)
    dx = 0.05
    mat = Material("neo_hookean", youngs_modulus=1e4, poissons_ratio=0.3)
    p = build_particles([
        (jittered_box(rng, (0.80, 0.8, 0.8), (6, 6, 6), dx / 2), mat, (2.0, 0.0, 0.0), dx / 2),
        (jittered_box(rng, (1.07, 0.8, 0.8), (6, 6, 6), dx / 2), mat, (-2.0, 0.0, 0.0), dx / 2),
    ])
    consts = _consts(dx)
    # a quad in the plane x = 1.0 (normal +x) and its twin facing -x, 1 mm apart
    V1 = np.array([[1.0, 0.5, 0.5], [1.0, 1.5, 0.5], [1.0, 1.5, 1.5], [1.0, 0.5, 1.5]], np.float32)
    V2 = V1 - np.array([0.001, 0, 0], np.float32)
    V = np.concatenate([V1, V2])
    T = np.array([[0, 1, 2], [0, 2, 3], [4, 6, 5], [4, 7, 6]], np.uint32)
    col = np.array([0, 0, 1, 1], np.uint32)
    gpu, ref = _pair(p, consts, _frame(V=V, T=T, col=col, g_a=(0, 0, 0), g_b=(0, 0, 0)))
    n, dt = 300, 1e-4
    assert gpu.step(n, dt, (0, 0, 0)) == (0, n)
    assert ref.step(n, dt, (0, 0, 0)) == 0
    out, exp = _check(gpu, ref, consts)
    left = np.arange(p.n) < p.n // 2
    assert out.positions[left, 0].max() < 1.0 and out.positions[~left, 0].min() > 0.999
    assert len(np.unique(out.collider_bits)) >= 3  # far, near-left, near-right
    gpu.close()


def test_frame_boundary_and_next_frame(cuda_lib, oracle_mod):
    """Stepping to the end of frame 0 leaves nothing pending; loading frame 1
    continues where the reference would; a substep outside the loaded frame
    fails like the reference's WrongFrameLoaded."""
    p = _falling_box()
    consts = _consts()
    V, T, col = _quad(0.45)
    gpu, ref = _pair(p, consts, _frame(0, V=V, T=T, col=col, g_b=(0, 0, -5)))
    dt = np.float32(2e-4)
    n0 = int(np.ceil((1.0 / FPS) / float(dt)))
    assert gpu.step(n0, float(dt), (0, 0, 0)) == (0, n0)
    assert ref.step(n0, float(dt), (0, 0, 0)) == 0
    assert gpu.time >= 1.0 / FPS and abs(gpu.time - ref.time) < 1e-12
    with pytest.raises(SvError):
        gpu.step(1, float(dt), (0, 0, 0))  # frame 0 still loaded
    fd1 = _frame(1, V=V, T=T, col=col, g_a=(0, 0, -5), g_b=(0, 0, -1))
    gpu.set_frame_input(fd1)
    ref.set_frame_input(fd1)
    assert gpu.step(60, float(dt), (0, 0, 0)) == (0, 60)
    assert ref.step(60, float(dt), (0, 0, 0)) == 0
    _check(gpu, ref, consts)
    gpu.close()


def test_moving_collider_pushes_particles(cuda_lib, oracle_mod):
    """A quad rising through frame 0 (vertex velocities from frames a and b)."""
    p = _falling_box(speed=0.0, z0=0.55)
    consts = _consts()
    V, T, col = _quad(0.45)
    Vb = V + np.array([0, 0, 0.2], np.float32)
    gpu, ref = _pair(p, consts, _frame(V=V, T=T, col=col, Vb=Vb, g_a=(0, 0, 0), g_b=(0, 0, 0)))
    n, dt = 300, 1e-4
    assert gpu.step(n, dt, (0, 0, 0)) == (0, n)
    assert ref.step(n, dt, (0, 0, 0)) == 0
    out, _ = _check(gpu, ref, consts)
    assert out.velocities[:, 2].max() > 0.5  # lifted
    gpu.close()


def test_adaptive_steps_with_a_collider(cuda_lib, oracle_mod):
    p = _falling_box()
    consts = _consts()
    V, T, col = _quad(0.45)
    gpu, ref = _pair(p, consts, _frame(V=V, T=T, col=col))
    status, done, t = gpu.step_adaptive(0.02, 1e-3, (0, 0, 0), time=0.0)
    rc, n_ref, t_ref, _ = ref.step_adaptive(0.0, 0.02, 1e-3, (0, 0, 0))
    assert (status, rc) == (0, 0) and done == n_ref
    assert abs(t - t_ref) <= 1e-6 * t_ref
    _check(gpu, ref, consts)
    gpu.close()
