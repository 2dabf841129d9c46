"""Known-answer cases ported from the reference's own unit tests.

Each function returns the grid/box of the reference test, the analytic input
and the analytic expected output, plus the tolerance the reference uses.
The same cases run against the CPU oracle (test_oracle_kat.py) and against
the GPU library (the known-answer tests of test_gpu_parity.py).

Arrays follow the reference layout: a scalar field is shaped (nx, ny, nz+1)
in C order (z fastest), a vector field (3, nx, ny, nz+1).
"""
import numpy as np

PI = np.pi


def grid(nx, ny, nz, lower, extent):
    dx = np.array(extent, dtype=np.float64) / np.array([nx, ny, nz], dtype=np.float64)
    x = lower[0] + np.arange(nx) * dx[0]
    y = lower[1] + np.arange(ny) * dx[1]
    z = lower[2] + np.arange(nz + 1) * dx[2]
    return np.meshgrid(x, y, z, indexing="ij")


def beltrami(nx, ny, nz, lower, extent, k=2.0, l=2.0, m=1.0):
    """Beltrami flow of unit-tests/test_vor2vel_1.f90:58-84 (and
    src/beltrami.f90:162-181): returns (vor, vel)."""
    X, Y, Z = grid(nx, ny, nz, lower, extent)
    alpha = np.sqrt(k * k + l * l + m * m)
    fk2l2 = 1.0 / (k * k + l * l)
    cosmz, sinmz = np.cos(m * Z), np.sin(m * Z)
    sinkxly, coskxly = np.sin(k * X + l * Y), np.cos(k * X + l * Y)
    u = fk2l2 * (k * m * sinmz - l * alpha * cosmz) * sinkxly
    v = fk2l2 * (l * m * sinmz + k * alpha * cosmz) * sinkxly
    w = cosmz * coskxly
    vel = np.stack([u, v, w])
    return alpha * vel, vel


def vor2vel_1():
    """unit-tests/test_vor2vel_1.f90: Beltrami k=l=2, m=1 on 32^3,
    [-pi/2, pi/2]^3, max-abs error < 1e-14."""
    nx = ny = nz = 32
    lower, extent = [-0.5 * PI] * 3, [PI] * 3
    vor, vel = beltrami(nx, ny, nz, lower, extent)
    return dict(nx=nx, ny=ny, nz=nz, lower=lower, extent=extent, vor=vor, vel=vel, atol=1.0e-14)


def vor2vel_2():
    """unit-tests/test_vor2vel_2.f90: f(z) = 2z - z^2 - z^3 flow, 32^3 on
    [-1/2,1/2]^2 x [0,1], tolerance 1.2e-2."""
    nx = ny = nz = 32
    lower, extent = [-0.5, -0.5, 0.0], [1.0, 1.0, 1.0]
    X, Y, Z = grid(nx, ny, nz, lower, extent)
    l = 2.0 * PI
    k = 2.0 * l
    klsq = k * k - l * l
    f = 2 * Z - Z ** 2 - Z ** 3
    dfdz = 2 - 2 * Z - 3 * Z ** 2
    d2fdz2 = -2 - 6 * Z
    sinkx, coskx = np.sin(k * X), np.cos(k * X)
    sinly, cosly = np.sin(l * Y), np.cos(l * Y)
    vel = np.stack([k * dfdz * coskx * sinly, -l * dfdz * sinkx * cosly, klsq * f * sinkx * sinly])
    vor = np.stack([l * (klsq * f + d2fdz2) * sinkx * cosly,
                    k * (d2fdz2 - klsq * f) * coskx * sinly,
                    -2.0 * k * l * dfdz * coskx * cosly])
    return dict(nx=nx, ny=ny, nz=nz, lower=lower, extent=extent, vor=vor, vel=vel, atol=1.2e-2)


def _mean_flow_case(eta_of_z, u_of_z, atol):
    nx = ny = nz = 32
    lower, extent = [-0.5, -0.5, 0.0], [1.0, 1.0, 1.0]
    X, Y, Z = grid(nx, ny, nz, lower, extent)
    zero = np.zeros_like(Z)
    vor = np.stack([zero, eta_of_z(Z), zero])
    vel = np.stack([u_of_z(Z), zero, zero])
    return dict(nx=nx, ny=ny, nz=nz, lower=lower, extent=extent, vor=vor, vel=vel, atol=atol)


def vor2vel_3():
    """unit-tests/test_vor2vel_3.f90: eta = 1 gives u = z - (zmin+zmax)/2."""
    return _mean_flow_case(lambda z: np.ones_like(z), lambda z: z - 0.5 * (0.0 + 1.0), 1.0e-15)


def vor2vel_4():
    """unit-tests/test_vor2vel_4.f90: eta = 2z gives u = z^2 - 1/3."""
    return _mean_flow_case(lambda z: 2.0 * z, lambda z: z ** 2 - 1.0 / 3.0, 1.0e-15)


def vor2vel_5():
    """unit-tests/test_vor2vel_5.f90: eta = 3z^2 gives u = z^3 - 1/4 (4e-6)."""
    return _mean_flow_case(lambda z: 3.0 * z ** 2, lambda z: z ** 3 - 0.25, 4.0e-6)


VOR2VEL_CASES = {"vor2vel_1": vor2vel_1, "vor2vel_2": vor2vel_2, "vor2vel_3": vor2vel_3,
                 "vor2vel_4": vor2vel_4, "vor2vel_5": vor2vel_5}


def diffz_cases():
    """unit-tests/test_diffz_1..4.f90: central_diffz on analytic fields."""
    out = {}
    X, Y, Z = grid(32, 32, 32, [0, 0, 0], [1, 1, 1])
    out["diffz_1"] = dict(nx=32, ny=32, nz=32, lower=[0, 0, 0], extent=[1, 1, 1],
                          f=Z.copy(), dfdz=np.ones_like(Z), atol=1.0e-14)
    lower, extent = [0.0, -0.5 * PI, 0.0], [PI, 2 * PI, 2 * PI]
    X, Y, Z = grid(16, 32, 32, lower, extent)
    ck, sl = np.cos(2.0 * X), np.sin(1.0 * Y)
    out["diffz_2"] = dict(nx=16, ny=32, nz=32, lower=lower, extent=extent,
                          f=Z * ck * sl, dfdz=ck * sl, atol=2.0e-14)
    out["diffz_3"] = dict(nx=16, ny=32, nz=32, lower=lower, extent=extent,
                          f=6 * Z + 3 * ck * sl * Z, dfdz=6 + 3 * ck * sl, atol=2.0e-13)
    X, Y, Z = grid(32, 32, 32, [0, 0, 0], [1, 1, 1])
    out["diffz_4"] = dict(nx=32, ny=32, nz=32, lower=[0, 0, 0], extent=[1, 1, 1],
                          f=1 - 3 * Z ** 2, dfdz=-6 * Z, atol=1.0e-1)
    return out


def diffxy_cases():
    """unit-tests/test_diffx.f90 (64x128x64, cos(4x)) and test_diffy.f90
    (128x64x64, cos(4y)) on [-pi,pi]^3.  The reference checks only
    (result - expected) < 1e-12 (one-sided); the port checks |.| < 1e-12."""
    lower, extent = [-PI] * 3, [2 * PI] * 3
    X, Y, Z = grid(64, 128, 64, lower, extent)
    cx = dict(nx=64, ny=128, nz=64, lower=lower, extent=extent, f=np.cos(4 * X),
              df=-4 * np.sin(4 * X), axis="x", atol=1.0e-12)
    X, Y, Z = grid(128, 64, 64, lower, extent)
    cy = dict(nx=128, ny=64, nz=64, lower=lower, extent=extent, f=np.cos(4 * Y),
              df=-4 * np.sin(4 * Y), axis="y", atol=1.0e-12)
    return {"diffx": cx, "diffy": cy}


def implicit_rk_reference(time_step):
    """unit-tests/test_implicit_rk.f90:62-94: with S = D = 1 held constant the
    integrating-factor RK4 step differs from the exact q E + (1-E) S/D by
    O(dt^5).  Returns (q0, exact) for q0 = 2."""
    e = np.exp(-time_step)
    return 2.0, 2.0 * e + (1.0 - e)


def if_rk4_constant(q0, s, d, dt):
    """The integrating-factor RK4 of src/stepper/impl_rk4.f90 applied to
    dq/dt = -d q + s with constant s and d (the scheme of
    unit-tests/test_implicit_rk.f90:106-239)."""
    dt2, dt3, dt6 = 0.5 * dt, dt / 3.0, dt / 6.0
    epq = np.exp(0.5 * d * dt)
    emq = 1.0 / epq
    qdi = q0
    q = (qdi + dt2 * s) * emq
    qdf = qdi + dt6 * s
    sqs = s * epq
    q = (qdi + dt2 * sqs) * emq
    qdf = qdf + dt3 * sqs
    emq = emq * emq
    sqs = s * epq
    q = (qdi + dt * sqs) * emq
    qdf = qdf + dt3 * sqs
    epq = epq * epq
    sqs = s * epq
    q = (qdf + dt6 * sqs) * emq
    return q
