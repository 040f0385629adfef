"""Initial states for the MHD step, in the reference layout.

u(5,nx,ny,nz) = (rho, m_x, m_y, m_z, E) and b(3,nx,ny,nz) face-centred on the
left faces, component fastest then i, j, k (Heterogeneous_MHD/C/array_definition.h:12-14).
All generators return flat float32 (or float64) numpy arrays ``(u, b)``.

The box has unit cell size, L = n along each axis, as in the reference driver
(tf = 4*nx, Heterogeneous_MHD/C/mhd.c:59).  E is built with the same face->centre
average of B that fluidx applies (Heterogeneous_MHD/C/fluidx.c:71-81), so a
uniform state is in discrete equilibrium.
"""
from __future__ import annotations

import numpy as np

GAMMA = 5.0 / 3.0


def _pack(rho, m, e, b, dtype):
    """rho,e: (nz,ny,nx); m,b: (3,nz,ny,nx) -> flat AoS u, b."""
    nz, ny, nx = rho.shape
    u = np.empty((nz, ny, nx, 5), dtype=np.float64)
    u[..., 0] = rho
    u[..., 1:4] = np.moveaxis(m, 0, -1)
    u[..., 4] = e
    bb = np.moveaxis(b, 0, -1)
    return (np.ascontiguousarray(u.astype(dtype)).ravel(),
            np.ascontiguousarray(bb.astype(dtype)).ravel())


def centred_b(b):
    """Face (left) -> cell centre average, b: (3,nz,ny,nx)."""
    return np.stack([(b[0] + np.roll(b[0], -1, axis=2)) / 2,
                     (b[1] + np.roll(b[1], -1, axis=1)) / 2,
                     (b[2] + np.roll(b[2], -1, axis=0)) / 2])


def _energy(rho, m, b, p):
    bc = centred_b(b)
    return p / (GAMMA - 1.0) + 0.5 * (m ** 2).sum(0) / rho + 0.5 * (bc ** 2).sum(0)


def alfven_x(n=32, amp=1e-3, rho0=1.0, p0=1.0, dtype=np.float32, ny=None, nz=None):
    """Linear Alfven wave along x on B0=(1,0,0): dv_y = A cos(2 pi x/L),
    dB_y = -A sqrt(rho) cos(2 pi x/L), x at cell centres (i+1/2).  b_y sits on
    y-faces at the x cell centre, so it is divergence-free exactly."""
    nx = n
    ny = n if ny is None else ny
    nz = n if nz is None else nz
    x = (np.arange(nx) + 0.5)
    ph = np.cos(2 * np.pi * x / nx)[None, None, :] * np.ones((nz, ny, 1))
    rho = np.full((nz, ny, nx), rho0)
    m = np.zeros((3, nz, ny, nx))
    m[1] = rho * amp * ph
    b = np.zeros((3, nz, ny, nx))
    b[0] = 1.0
    b[1] = -amp * np.sqrt(rho0) * ph
    e = _energy(rho, m, b, p0)
    return _pack(rho, m, e, b, dtype)


def _edge_potential_curl(ax, ay, az):
    """Discrete curl of an edge-centred vector potential onto left faces.

    A_x lives at (i+1/2, j, k), A_y at (i, j+1/2, k), A_z at (i, j, k+1/2)
    (arrays indexed [k, j, i]); b_x at (i, j+1/2, k+1/2) etc.  The result has
    zero discrete divergence b1(i+1)-b1(i)+b2(j+1)-b2(j)+b3(k+1)-b3(k)."""
    dyz = lambda a, axis: np.roll(a, -1, axis=axis) - a
    bx = dyz(az, 1) - dyz(ay, 0)
    by = dyz(ax, 0) - dyz(az, 2)
    bz = dyz(ay, 2) - dyz(ax, 1)
    return np.stack([bx, by, bz])


def alfven_oblique(n=128, kvec=(1, 1, 1), amp=1e-3, rho0=1.0, p0=1.0, dtype=np.float32,
                   ny=None, nz=None):
    """Linear Alfven wave with wave vector k = (kvec_i 2pi/L_i) and B0 = khat.

    The perturbation direction is e1 = normalised (khat x z) (or khat x x when
    khat is parallel to z); dv = A cos(k.x) e1 at cell centres and
    dB = -A sqrt(rho) cos(k.x) e1 from a staggered vector potential, so the
    face field is divergence-free to round-off.  ny, nz default to n (cubic);
    on a non-cubic box the wave stays periodic (kvec integer per axis)."""
    nx = n
    ny = n if ny is None else ny
    nz = n if nz is None else nz
    kv = np.asarray(kvec, dtype=np.float64) * 2 * np.pi / np.array([nx, ny, nz], dtype=np.float64)
    kh = kv / np.linalg.norm(kv)
    ref = np.array([0.0, 0.0, 1.0]) if abs(kh[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    e1 = np.cross(kh, ref)
    e1 /= np.linalg.norm(e1)
    kk, jj, ii = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")

    def phase(ox, oy, oz):
        return kv[0] * (ii + ox) + kv[1] * (jj + oy) + kv[2] * (kk + oz)

    rho = np.full((nz, ny, nx), rho0)
    m = rho * amp * np.cos(phase(0.5, 0.5, 0.5))[None] * e1[:, None, None, None]
    # dB = -amp*sqrt(rho)*cos(k.x) e1 = curl(a sin(k.x)), a = -amp*sqrt(rho)*(e1 x k)/|k|^2
    a = -amp * np.sqrt(rho0) * np.cross(e1, kv) / np.dot(kv, kv)
    ax = a[0] * np.sin(phase(0.5, 0.0, 0.0))
    ay = a[1] * np.sin(phase(0.0, 0.5, 0.0))
    az = a[2] * np.sin(phase(0.0, 0.0, 0.5))
    b = _edge_potential_curl(ax, ay, az)
    b += kh[:, None, None, None]
    e = _energy(rho, m, b, p0)
    return _pack(rho, m, e, b, dtype)


def _spectral_field(r, nx, ny, nz, slope):
    """Real Gaussian random field on (nz, ny, nx) whose Fourier amplitudes go as
    |k|^slope (k in units of the longest axis' fundamental; no k = 0 mode)."""
    lmax = float(max(nx, ny, nz))
    kz = np.fft.fftfreq(nz) * nz * (lmax / nz)
    ky = np.fft.fftfreq(ny) * ny * (lmax / ny)
    kx = np.fft.rfftfreq(nx) * nx * (lmax / nx)
    kk = np.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2)
    amp = np.zeros_like(kk)
    amp[kk > 0] = kk[kk > 0] ** slope
    noise = np.fft.rfftn(r.standard_normal((nz, ny, nx)))
    return np.fft.irfftn(noise * amp, s=(nz, ny, nx), axes=(0, 1, 2))


def turbulence(nx, ny=None, nz=None, seed=0, mach=0.5, b_mean=0.3, db_rms=None, v_rms=None,
               rho0=1.0, p0=1.0, dtype=np.float32):
    """Seeded Gaussian-random turbulent start.

    Velocity: each component a Gaussian random field with Fourier amplitudes
    |k|^-2 (shell energy spectrum E(k) ~ k^-2), scaled to rms |v| = mach * c_s
    (c_s = sqrt(gamma p0/rho0)) unless v_rms is given.  Field: B = B_mean x +
    curl A, A a vector potential with Fourier amplitudes |k|^-2.5 (E_A(k) ~
    k^-3) on the cell edges, so the face field is divergence-free to round-off;
    the fluctuation is scaled to rms |dB| = db_rms (default: the rms |v|).
    rho = rho0, p = p0 uniform."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    r = np.random.default_rng(seed)
    v = np.stack([_spectral_field(r, nx, ny, nz, -2.0) for _ in range(3)])
    target_v = mach * np.sqrt(GAMMA * p0 / rho0) if v_rms is None else v_rms
    v *= target_v / np.sqrt((v ** 2).sum(0).mean())
    a = [_spectral_field(r, nx, ny, nz, -2.5) for _ in range(3)]
    db = _edge_potential_curl(*a)
    target_b = target_v if db_rms is None else db_rms
    db *= target_b / np.sqrt((db ** 2).sum(0).mean())
    db[0] += b_mean
    rho = np.full((nz, ny, nx), rho0)
    m = rho[None] * v
    e = _energy(rho, m, db, p0)
    return _pack(rho, m, e, db, dtype)


def ensemble_specs(nbox=64, seed=0, sizes=(32, 48, 64, 96, 128), amp_range=(1e-4, 1e-1)):
    """The draws of ensemble() without building the states: a list of dicts
    {dims: (nx, ny, nz), kind, amp, seed}, in box order."""
    r = np.random.default_rng(seed)
    out = []
    for _ in range(nbox):
        dims = tuple(int(x) for x in r.choice(sizes, size=3))
        amp = float(np.exp(r.uniform(np.log(amp_range[0]), np.log(amp_range[1]))))
        kind = "alfven" if r.random() < 0.5 else "turbulent"
        bseed = int(r.integers(0, 2 ** 31 - 1))
        out.append({"dims": dims, "kind": kind, "amp": amp, "seed": bseed})
    return out


def ensemble_dims(nbox=64, seed=0, sizes=(32, 48, 64, 96, 128), amp_range=(1e-4, 1e-1)):
    """The box sizes of ensemble(), cheaply."""
    return [e["dims"] for e in ensemble_specs(nbox, seed, sizes, amp_range)]


def ensemble(nbox=64, seed=0, sizes=(32, 48, 64, 96, 128), amp_range=(1e-4, 1e-1),
             dtype=np.float32):
    """The batched-ensemble workload: nbox independent periodic boxes whose
    sizes along each axis are drawn from `sizes` by seed (non-cubic, uneven),
    each a linear Alfven wave on the box diagonal (kvec = (1,1,1) per axis) or a
    turbulent start (turbulence(), rms |v| = rms |dB| = the amplitude), with an
    amplitude drawn log-uniformly from amp_range.

    Returns a list of dicts {dims: (nx, ny, nz), kind, amp, seed, u, b}."""
    out = []
    for e in ensemble_specs(nbox, seed, sizes, amp_range):
        dims, amp = e["dims"], e["amp"]
        if e["kind"] == "alfven":
            u, b = alfven_oblique(dims[0], amp=amp, ny=dims[1], nz=dims[2], dtype=dtype)
        else:
            u, b = turbulence(*dims, seed=e["seed"], v_rms=amp, db_rms=amp, dtype=dtype)
        out.append(dict(e, u=u, b=b))
    return out


def blast(n=256, r0=0.1, p_in=100.0, p_out=0.1, rho0=1.0, b0=(10.0 / np.sqrt(2.0), 10.0 / np.sqrt(2.0), 0.0),
          dtype=np.float32, ny=None, nz=None):
    """Spherical MHD blast: gas pressure p_in inside radius r0*L of the box
    centre and p_out outside, rho = rho0 and v = 0 everywhere, uniform
    B = b0 (default (1,1,0)/sqrt(2)*10: beta = 2 p_out/B^2 = 0.002 outside).
    L = n (unit cells); the radius is measured between cell centres."""
    nx = n
    ny = n if ny is None else ny
    nz = n if nz is None else nz
    kk, jj, ii = np.meshgrid(np.arange(nz) + 0.5, np.arange(ny) + 0.5, np.arange(nx) + 0.5, indexing="ij")
    r = np.sqrt((ii - nx / 2) ** 2 + (jj - ny / 2) ** 2 + (kk - nz / 2) ** 2)
    rho = np.full((nz, ny, nx), rho0)
    p = np.where(r < r0 * nx, p_in, p_out)
    m = np.zeros((3, nz, ny, nx))
    b = np.broadcast_to(np.asarray(b0, dtype=np.float64)[:, None, None, None], (3, nz, ny, nx)).copy()
    e = _energy(rho, m, b, p)
    return _pack(rho, m, e, b, dtype)


FORTRAN_ICS = ("sound", "cp_alfven", "alfven", "magnetic", "magnetosonic", "oblique")


def fortran_ic(kind, nx, ny=1, nz=None):
    """The analytic initial states of the Fortran original's init
    (OpenMP/mhd.f90:130-247), restated in float32 (its default real kind):
    1-based x index i, phase 2*3.14159*i/nx in float, cshift(a,-1,dim)
    = roll by +1 along dim.

      sound:        rho = 1 + 1e-4 sin, m_x = 1e-4 sin on the (j,k) = (1,1) line,
                    p0 = 3/5, B = (1,0,0)            (mhd.f90:136-146)
      cp_alfven:    circularly polarised Alfven wave, amplitude 0.1, B0 = x
                                                      (mhd.f90:147-162)
      alfven:       linear Alfven wave, m_y = 0.1 sin, b_y = -m_y averaged
                    with its x-1 neighbour            (mhd.f90:164-179)
      magnetic:     m_x = 1e-3 sin, b_y = 1 + m_x, rho = b_y (mhd.f90:180-192)
      magnetosonic: p0 = 3/10, b_y = (1 + m_x)/sqrt 2, rho = 1 + m_x,
                    m_x = 1e-4 sin                    (mhd.f90:193-206)
      oblique:      the wave along (1,0,1) that the original ends on
                                                      (mhd.f90:222-246)
    Returns flat float32 (u, b) in the reference layout."""
    f32 = np.float32
    nz = nx if nz is None else nz
    if kind not in FORTRAN_ICS:
        raise ValueError(f"unknown initial state {kind!r}; one of {FORTRAN_ICS}")
    u = np.zeros((5, nz, ny, nx), dtype=f32)      # [field, k, j, i]
    b = np.zeros((3, nz, ny, nx), dtype=f32)
    two_pi = f32(2) * f32(3.14159)
    ph = (two_pi * np.arange(1, nx + 1, dtype=f32) / f32(nx)).astype(f32)    # along x
    sin_x, cos_x = np.sin(ph).astype(f32), np.cos(ph).astype(f32)
    half = f32(2)

    def ke(u):
        return ((u[1] ** 2 + u[2] ** 2 + u[3] ** 2) / u[0] / half).astype(f32)

    def me(b):
        return ((b[0] ** 2 + b[1] ** 2 + b[2] ** 2) / half).astype(f32)

    if kind == "sound":
        p0 = f32(3.0) / f32(5.0)
        b[0] = 1
        u[0] = 1
        u[4] = f32(1.5) * p0
        u[1, 0, 0, :] = f32(0.0001) * sin_x
        u[0, 0, 0, :] = u[0, 0, 0, :] + u[1, 0, 0, :]
        u[4] = u[4] + me(b) + (u[1] ** 2 / u[0] / half).astype(f32)
        u[4, 0, 0, :] = u[4, 0, 0, :] + p0 * u[1, 0, 0, :] * f32(5.0) / f32(3.0) / (f32(2.0) / f32(3.0))
    elif kind == "cp_alfven":
        b[0] = 1
        u[0] = 1
        u[4] = f32(0.1)
        u[2] = f32(0.1) * sin_x
        u[3] = f32(0.1) * cos_x
        b[1] = -u[2]
        b[2] = -u[3]
        b[1] = (b[1] + np.roll(b[1], 1, axis=1)) / half      # cshift(.,-1,2): along y
        b[2] = (b[2] + np.roll(b[2], 1, axis=0)) / half      # cshift(.,-1,3): along z
        u[4] = u[4] + me(b) + ke(u)
    elif kind == "alfven":
        b[0] = 1
        u[0] = 1
        u[4] = f32(0.001)
        u[2] = f32(0.1) * sin_x
        b[1] = -u[2]
        b[1] = (b[1] + np.roll(b[1], 1, axis=2)) / half      # cshift(.,-1,1): along x
        u[4] = u[4] + me(b) + (u[2] ** 2 / u[0] / half).astype(f32)
    elif kind == "magnetic":
        b[1] = 1
        u[0] = 1
        u[4] = f32(0.000000001)
        u[1] = f32(0.001) * sin_x
        b[1] = b[1] + u[1]
        u[0] = b[1]
        u[4] = u[4] + me(b) + ke(u)
    elif kind == "magnetosonic":
        p0 = f32(3.0) / f32(5.0) / f32(2.0)
        r2 = f32(np.sqrt(f32(2.0)))
        b[1] = f32(1.0) / r2
        u[0] = 1
        u[4] = p0 * f32(1.5)
        u[1] = f32(0.0001) * sin_x
        b[1] = b[1] + u[1] / r2
        u[0] = u[0] + u[1]
        u[4] = u[4] + me(b) + ke(u)
        u[4] = u[4] + p0 * u[1] * f32(5.0) / f32(3.0) / (f32(2.0) / f32(3.0))
    else:  # oblique
        r2 = f32(np.sqrt(f32(2.0)))
        phk = (two_pi * np.arange(1, nz + 1, dtype=f32) / f32(nz)).astype(f32)
        p = (ph[None, None, :] + phk[:, None, None]).astype(f32) * np.ones((1, ny, 1), dtype=f32)
        sp, cp = np.sin(p).astype(f32), np.cos(p).astype(f32)
        u[0] = 1
        u[2] = f32(-0.1) * cp
        u[1] = f32(-0.1) * sp / r2
        u[3] = f32(0.1) * sp / r2
        b[1] = f32(0.1) * cp
        b[0] = (f32(1.0) + f32(0.1) * sp) / r2
        b[2] = (f32(1.0) - f32(0.1) * sp) / r2
        u[4] = f32(1.5) + f32(0.01)
    uu = np.ascontiguousarray(np.moveaxis(u, 0, -1)).ravel()
    bb = np.ascontiguousarray(np.moveaxis(b, 0, -1)).ravel()
    return uu.astype(np.float32), bb.astype(np.float32)


def random_state(nx, ny, nz, seed=0, dtype=np.float32, amp=0.3, bmean=(0.3, 0.1, -0.2)):
    """Seeded random but physical state (positive density and pressure) used by
    the per-subroutine parity tests."""
    r = np.random.default_rng(seed)
    rho = 1.0 + 0.2 * r.random((nz, ny, nx))
    m = amp * r.standard_normal((3, nz, ny, nx))
    b = 0.5 * r.standard_normal((3, nz, ny, nx)) + np.asarray(bmean)[:, None, None, None]
    p = 1.0 + 0.1 * r.random((nz, ny, nx))
    e = _energy(rho, m, b, p)
    return _pack(rho, m, e, b, dtype)


def div_b(b, nx, ny, nz):
    """max |b1(i+1)-b1(i)+b2(j+1)-b2(j)+b3(k+1)-b3(k)| in float64 (left faces)."""
    bb = np.asarray(b, dtype=np.float64).reshape(nz, ny, nx, 3)
    d = (np.roll(bb[..., 0], -1, 2) - bb[..., 0] + np.roll(bb[..., 1], -1, 1) - bb[..., 1]
         + np.roll(bb[..., 2], -1, 0) - bb[..., 2])
    return float(np.abs(d).max())


def totals(u, nx, ny, nz):
    """FP64 sums of rho, m_x, m_y, m_z, E."""
    return np.asarray(u, dtype=np.float64).reshape(-1, 5).sum(0)
