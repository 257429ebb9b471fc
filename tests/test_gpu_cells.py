"""Spatially inhomogeneous use: per-cell collision steps fed from a transport
step (CellSolver, edb_cells_transport_x_device).

Tolerances
  Transport, integer shifts: bit-exact (a periodic roll of each velocity slice).
  Transport, fractional shifts: against the same rule in numpy <= 1e-14 of
    max|f| (the kernel may fuse the interpolation into one FMA); every velocity
    slice's total kept to 1e-13 relative; no negative values.
  collide: equals load -> step -> read of a BatchSolver to 1e-12 relative L2.
  Strang steps: against a CPU composition (the same transport in numpy, the
    oracle's FP64 RK4 collision step per cell) <= 2e-6 of max|f| (the GPU's
    Q-hat is FP32 with compensated sums); with conservative collisions the
    total mass, momentum and energy over all cells are kept to 1e-10
    relative (momentum relative to sqrt(mass * energy)).
"""
import numpy as np
import pytest

from oracle.oracle import INDEX_ALIASED

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def edb():
    import entropydecreaseboltzmann_gb300 as e

    return e


def transport_np(f, N, R, Lx, dt):
    """The transport rule of edb_cells_transport_x_device, in numpy."""
    C = f.shape[0]
    h = 2.0 * R / N
    dx = Lx / C
    v1 = -R + h * np.arange(N)
    out = np.empty_like(f)
    g = f.reshape(C, N, N * N)
    o = out.reshape(C, N, N * N)
    for i1 in range(N):
        s = v1[i1] * dt / dx
        n = int(np.floor(s))
        th = s - n
        a = np.roll(g[:, i1, :], n, axis=0)
        b = np.roll(g[:, i1, :], n + 1, axis=0)
        o[:, i1, :] = (1.0 - th) * a + th * b
    return out


def sod_like(N, R, C, seed=3):
    """Left half: a dense cold Maxwellian, right half: a dilute hot one, with
    seeded small drifts (every cell mass-normalised to its density)."""
    from entropydecreaseboltzmann_gb300 import data

    rng = np.random.default_rng(seed)
    f = np.empty((C, N ** 3))
    for c in range(C):
        left = c < C // 2
        rho, T = (1.0, 0.8) if left else (0.4, 1.3)
        u = rng.uniform(-0.3, 0.3, size=3)
        m = data.maxwellian(N, R, 1.0, u, T)
        f[c] = rho * m / data.mass(m, N, R)
    return f


def moments(f, N, R):
    from entropydecreaseboltzmann_gb300 import data

    h, X, Y, Z = data.grid(N, R)
    w = h ** 3
    tot = f.sum(axis=0)
    return np.array([w * tot.sum(), w * (tot * X).sum(), w * (tot * Y).sum(),
                     w * (tot * Z).sum(), w * (tot * (X * X + Y * Y + Z * Z)).sum()])


def test_transport_integer_and_fractional_shifts(edb):
    import torch

    N, R, C = 8, 6.0, 10
    h = 2.0 * R / N
    f = sod_like(N, R, C)
    d_f = torch.from_numpy(f).cuda()
    d_o = torch.empty_like(d_f)
    q = edb.QCalculator(N, 0, L=R, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    # dx = h dt: v1 dt / dx = v1 / h, an integer for every v1 on the grid (h =
    # 1.5, dt = 0.5: every quantity is exact in binary, so theta = 0 exactly)
    dt = 0.5
    cells = edb.CellSolver(q, C, R, Lx=C * h * dt, dt=dt)
    cells.transport(d_f, d_o, dt)
    torch.cuda.synchronize()
    assert np.array_equal(d_o.cpu().numpy(), transport_np(f, N, R, C * h * dt, dt))
    # fractional shifts
    Lx, dt = 3.7, 0.013
    cells = edb.CellSolver(q, C, R, Lx=Lx, dt=dt)
    cells.transport(d_f, d_o, dt)
    torch.cuda.synchronize()
    got = d_o.cpu().numpy()
    assert np.max(np.abs(got - transport_np(f, N, R, Lx, dt))) <= 1e-14 * np.max(np.abs(f))
    assert got.min() >= 0.0
    np.testing.assert_allclose(got.sum(axis=0), f.sum(axis=0), rtol=1e-13, atol=0)


def test_collide_equals_batch_solver(edb):
    import torch

    N, R, C = 12, 6.0, 6
    f = sod_like(N, R, C)
    q = edb.QCalculator(N, 0, L=R, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    cells = edb.CellSolver(q, C, R, Lx=1.0, dt=0.01)
    d_f = torch.from_numpy(f).cuda()
    cells.collide(d_f, nsteps=3)
    torch.cuda.synchronize()
    b = edb.BatchSolver(q, C, R, edb.SCHEME_RK4, 0.01)
    b.load(f)
    b.step(3)
    want = b.read(real=True)
    got = d_f.cpu().numpy()
    assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)


def test_strang_steps_match_cpu_composition_and_conserve(edb, oracle):
    import torch

    N, R, C, Lx, dt, steps = 12, 6.0, 8, 2.0, 0.01, 2
    f0 = sod_like(N, R, C)
    q = edb.QCalculator(N, 0, L=R, filter=False, index_mode=INDEX_ALIASED)
    q.genB()
    cells = edb.CellSolver(q, C, R, Lx=Lx, dt=dt)
    d_f = torch.from_numpy(f0).cuda()
    d_t = torch.empty_like(d_f)
    for _ in range(steps):
        cells.strang_step(d_f, d_t)
    torch.cuda.synchronize()
    got = d_f.cpu().numpy()
    # the same composition on the CPU: numpy transport, the oracle's FP64 RK4
    # collision step (one step: TEnd = dt / 2)
    f = f0.copy()
    for _ in range(steps):
        f = transport_np(f, N, R, Lx, 0.5 * dt)
        for c in range(C):
            Fh, _, _, _ = oracle.run(N, R, "RK4", 0.0, 0.5 * dt, dt, fix=False, F0=f[c],
                                     mode=INDEX_ALIASED, Rb=R, filter=False)
            f[c] = np.fft.ifftn(Fh.reshape(N, N, N)).real.reshape(-1)
        f = transport_np(f, N, R, Lx, 0.5 * dt)
    assert np.max(np.abs(got - f)) <= 2e-6 * np.max(np.abs(f))
    # conservative collisions: the totals over all cells stay put
    cons = edb.CellSolver(q, C, R, Lx=Lx, dt=dt, conserve=True)
    d_f = torch.from_numpy(f0).cuda()
    for _ in range(3):
        cons.strang_step(d_f, d_t)
    torch.cuda.synchronize()
    m0, m1 = moments(f0, N, R), moments(d_f.cpu().numpy(), N, R)
    scale = np.array([m0[0], np.sqrt(m0[0] * m0[4]), np.sqrt(m0[0] * m0[4]),
                      np.sqrt(m0[0] * m0[4]), m0[4]])
    assert np.max(np.abs(m1 - m0) / scale) <= 1e-10
