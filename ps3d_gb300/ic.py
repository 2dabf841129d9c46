"""Initial conditions: the reference's Beltrami flow plus a seeded
perturbation of the spectral vorticity.

The Beltrami vorticity is src/beltrami.f90:162-181 evaluated on the grid
points x = lower + i dx (both walls included, beltrami.f90:141-160).  The
perturbation has no reference counterpart: Gaussian coefficients with a
K^-2 envelope, K = |(k, l, m)|, placed in the interior sine modes of the
mixed-spectral vorticity (boundary rows zero), from numpy's PCG64 generator
seeded with `seed`, rescaled so that its grid rms (Parseval) is
`amplitude * |omega|_rms` of the Beltrami field.  The first vor2vel of a run
projects the sum onto a solenoidal field (inversion.f90:34-76).
"""
import numpy as np

BELTRAMI_BOX = dict(lower=(0.0, 0.0, -0.5 * np.pi), extent=(2.0 * np.pi, 2.0 * np.pi, np.pi))


def beltrami_vorticity(nx, ny, nz, lower, extent, k=2, l=2, m=1):
    """(3, nx, ny, nz+1) FP64 physical vorticity of the Beltrami flow."""
    kk, ll, mm = float(k), float(l), float(m)
    alpha = np.sqrt(kk ** 2 + ll ** 2 + mm ** 2)
    fk2l2 = alpha / float(k * k + l * l)
    dx = np.array(extent, dtype=np.float64) / np.array([nx, ny, nz], dtype=np.float64)
    x = lower[0] + dx[0] * np.arange(nx, dtype=np.float64)
    y = lower[1] + dx[1] * np.arange(ny, dtype=np.float64)
    z = lower[2] + dx[2] * np.arange(nz + 1, dtype=np.float64)
    cosmz, sinmz = np.cos(mm * z), np.sin(mm * z)
    phase = kk * x[:, None] + ll * y[None, :]
    sinkxly, coskxly = np.sin(phase), np.cos(phase)
    out = np.empty((3, nx, ny, nz + 1))
    g1 = fk2l2 * (kk * mm * sinmz - ll * alpha * cosmz)
    g2 = fk2l2 * (ll * mm * sinmz + kk * alpha * cosmz)
    g3 = alpha * cosmz
    np.multiply(sinkxly[:, :, None], g1[None, None, :], out=out[0])
    np.multiply(sinkxly[:, :, None], g2[None, None, :], out=out[1])
    np.multiply(coskxly[:, :, None], g3[None, None, :], out=out[2])
    return out


def wavenumbers(nx, ny, nz, extent):
    """rkx, rky (Hermitian slot order, sta3dfft.f90:96-115), rkz (deriv1d.f90)."""
    def horiz(n, L):
        r = np.zeros(n)
        h = n // 2
        for kk in range(1, h):
            r[kk] = r[n - kk] = 2.0 * np.pi * kk / L
        r[h] = np.pi * n / L
        return r
    return horiz(nx, extent[0]), horiz(ny, extent[1]), np.pi * np.arange(nz + 1) / extent[2]


def perturbation(nx, ny, nz, extent, seed, amplitude, vor_rms):
    """(3, nx, ny, nz+1) mixed-spectral perturbation (see module docstring)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rkx, rky, rkz = wavenumbers(nx, ny, nz, extent)
    K2 = rkx[:, None, None] ** 2 + rky[None, :, None] ** 2 + rkz[None, None, :] ** 2
    env = np.zeros_like(K2)
    np.divide(1.0, K2, out=env, where=K2 > 0)          # K^-2 envelope
    env[:, :, 0] = 0.0
    env[:, :, nz] = 0.0
    env[nx // 2, :, :] = 0.0                            # no Nyquist modes
    env[:, ny // 2, :] = 0.0
    p = rng.standard_normal((3, nx, ny, nz + 1)) * env[None]
    # grid mean square by Parseval: Hermitian slots other than 0 and n/2
    # carry weight 2 in each horizontal direction; the sine transform is
    # orthonormal over the nz-1 interior levels
    wx = np.full(nx, 2.0); wx[0] = 1.0; wx[nx // 2] = 1.0
    wy = np.full(ny, 2.0); wy[0] = 1.0; wy[ny // 2] = 1.0
    w = wx[:, None, None] * wy[None, :, None]
    ms = float(np.sum(w[None] * p * p)) / (nx * ny * (nz + 1))
    scale = amplitude * vor_rms / np.sqrt(ms) if ms > 0 else 0.0
    p *= scale
    return p


def beltrami_plus_perturbation(nx, ny, nz, seed=0, amplitude=1.0e-3, lower=None, extent=None):
    """Physical Beltrami vorticity and the matching spectral perturbation,
    on the box (2pi, 2pi, pi) with lower z = -pi/2 unless given."""
    lower = BELTRAMI_BOX["lower"] if lower is None else lower
    extent = BELTRAMI_BOX["extent"] if extent is None else extent
    vor = beltrami_vorticity(nx, ny, nz, lower, extent)
    rms = float(np.sqrt(np.mean(np.sum(vor * vor, axis=0))))
    pert = perturbation(nx, ny, nz, extent, seed, amplitude, rms)
    return vor, pert


def beltrami_plus_perturbation_slabs(nx, ny, nz, seed=0, amplitude=1.0e-3, lower=None, extent=None):
    """Memory-lean variant for very large grids (1024^3: 26 GB per vector
    field): the same Beltrami field and the same perturbation recipe, built
    one x-slab at a time.  The Gaussian coefficients of slab ix come from
    PCG64 seeded with (seed, ix), so for a given seed the field differs from
    `beltrami_plus_perturbation`'s; host memory is the two output arrays plus
    one slab."""
    lower = BELTRAMI_BOX["lower"] if lower is None else lower
    extent = BELTRAMI_BOX["extent"] if extent is None else extent
    vor = np.empty((3, nx, ny, nz + 1))
    kk, ll, mm = 2.0, 2.0, 1.0
    alpha = np.sqrt(kk ** 2 + ll ** 2 + mm ** 2)
    fk2l2 = alpha / (kk * kk + ll * ll)
    dx = np.array(extent, dtype=np.float64) / np.array([nx, ny, nz], dtype=np.float64)
    y = lower[1] + dx[1] * np.arange(ny, dtype=np.float64)
    z = lower[2] + dx[2] * np.arange(nz + 1, dtype=np.float64)
    cosmz, sinmz = np.cos(mm * z), np.sin(mm * z)
    g = (fk2l2 * (kk * mm * sinmz - ll * alpha * cosmz), fk2l2 * (ll * mm * sinmz + kk * alpha * cosmz),
         alpha * cosmz)
    sq = 0.0
    for ix in range(nx):
        phase = kk * (lower[0] + dx[0] * ix) + ll * y
        s, c = np.sin(phase), np.cos(phase)
        vor[0, ix] = s[:, None] * g[0][None, :]
        vor[1, ix] = s[:, None] * g[1][None, :]
        vor[2, ix] = c[:, None] * g[2][None, :]
        sq += float(np.sum(vor[:, ix] * vor[:, ix]))
    rms = np.sqrt(sq / (nx * ny * (nz + 1)))
    rkx, rky, rkz = wavenumbers(nx, ny, nz, extent)
    wy = np.full(ny, 2.0); wy[0] = 1.0; wy[ny // 2] = 1.0
    pert = np.empty((3, nx, ny, nz + 1))
    ms = 0.0
    for ix in range(nx):
        K2 = rkx[ix] ** 2 + rky[:, None] ** 2 + rkz[None, :] ** 2
        env = np.zeros_like(K2)
        np.divide(1.0, K2, out=env, where=K2 > 0)
        env[:, 0] = 0.0
        env[:, nz] = 0.0
        env[ny // 2, :] = 0.0
        if ix == nx // 2:
            env[:] = 0.0
        rng = np.random.Generator(np.random.PCG64([seed, ix]))
        pert[:, ix] = rng.standard_normal((3, ny, nz + 1)) * env[None]
        wx = 1.0 if ix in (0, nx // 2) else 2.0
        ms += wx * float(np.sum(wy[None, :, None] * pert[:, ix] * pert[:, ix]))
    ms /= nx * ny * (nz + 1)
    scale = amplitude * rms / np.sqrt(ms) if ms > 0 else 0.0
    for ix in range(nx):
        pert[:, ix] *= scale
    return vor, pert


def kolmogorov_spectral_vorticity(nx, ny, nz, extent, seed=0):
    """(3, nx, ny, nz+1) seeded random mixed-spectral vorticity for the
    standalone vor2vel / diffz workloads: amplitude K^(-5/3), K = |(k, l, m)|
    from the reference's wavenumber tables (zero at K = 0), with uniform
    random phases.  In each horizontal direction a mode k has a cosine slot
    k and a sine slot n-k of the Hermitian layout (stafft.f90:55-58); the
    slot pair of mode k in x (and likewise in y) takes cos(phi), sin(phi) of
    a phase phi drawn uniformly in [0, 2pi) per component, mode and level
    (PCG64(seed)), and the coefficient is the product of the x and y
    factors.  Every level is filled, the wall rows (semi-spectral boundary
    values) included.  Normalised to unit rms over the stored values."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rkx, rky, rkz = wavenumbers(nx, ny, nz, extent)
    K2 = rkx[:, None, None] ** 2 + rky[None, :, None] ** 2 + rkz[None, None, :] ** 2
    amp = np.zeros_like(K2)
    np.power(K2, -5.0 / 6.0, out=amp, where=K2 > 0)

    def slots(n):
        j = np.arange(n)
        mode = np.where(j <= n // 2, j, n - j)
        return mode, j > n // 2

    mx, sx = slots(nx)
    my, sy = slots(ny)
    phx = rng.uniform(0.0, 2.0 * np.pi, size=(3, nx // 2 + 1, ny // 2 + 1, nz + 1))
    phy = rng.uniform(0.0, 2.0 * np.pi, size=(3, nx // 2 + 1, ny // 2 + 1, nz + 1))
    ax = phx[:, mx[:, None], my[None, :], :]
    ay = phy[:, mx[:, None], my[None, :], :]
    fx = np.where(sx[None, :, None, None], np.sin(ax), np.cos(ax))
    fy = np.where(sy[None, None, :, None], np.sin(ay), np.cos(ay))
    out = amp[None] * fx * fy
    out /= np.sqrt(np.mean(out * out))
    return out


def grid(nx, ny, nz, lower, extent):
    """Grid coordinates x (nx), y (ny), z (nz+1) of the reference's nodes."""
    dx = np.array(extent, dtype=np.float64) / np.array([nx, ny, nz], dtype=np.float64)
    return (lower[0] + dx[0] * np.arange(nx), lower[1] + dx[1] * np.arange(ny),
            lower[2] + dx[2] * np.arange(nz + 1))


def stratified_buoyancy(nx, ny, nz, lower, extent, bfsq=1.0, amplitude=1.0e-2, seed=0, kmax=3):
    """(nx, ny, nz+1) total physical buoyancy: the basic state N^2 z plus a
    perturbation (no reference counterpart; the reference reads its buoyancy
    from a NetCDF file): a sum of modes cos(k x + l y + phase) sin(j pi (z -
    lower_z) / L_z) with |k|, |l| <= kmax horizontal and 1 <= j <= kmax
    vertical wave numbers, Gaussian amplitudes from PCG64(seed), rescaled so
    that its grid rms is amplitude * N^2 * L_z.  The perturbation vanishes on
    the walls, so calculate_basic_reference_state recovers N^2 exactly."""
    rng = np.random.Generator(np.random.PCG64(seed))
    x, y, z = grid(nx, ny, nz, lower, extent)
    zeta = (z - lower[2]) / extent[2]
    pert = np.zeros((nx, ny, nz + 1))
    for k in range(0, kmax + 1):
        for l in range(-kmax, kmax + 1):
            if k == 0 and l <= 0:
                continue
            phase = 2.0 * np.pi * (k * (x[:, None] - lower[0]) / extent[0] + l * (y[None, :] - lower[1]) / extent[1])
            for j in range(1, kmax + 1):
                a, ph = rng.standard_normal(), rng.uniform(0.0, 2.0 * np.pi)
                pert += a * np.cos(phase + ph)[:, :, None] * np.sin(j * np.pi * zeta)[None, None, :]
    rms = np.sqrt(np.mean(pert ** 2))
    pert *= amplitude * bfsq * extent[2] / rms
    return bfsq * z[None, None, :] + pert
