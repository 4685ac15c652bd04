"""Seeded synthetic inputs for the analysis workloads.

No public benchmark data is involved: every case is generated from numpy
PCG64 streams seeded as ``20261203 + 100 * case + stream``.

* ``global_etkf_grid``  64 x 64 single-variable grid, Gaussian random field
  with squared-exponential covariance (length 8 cells, sigma 1); members =
  truth + independent draws of the same field; point obs at distinct
  uniformly drawn cells, IDW4 (reference) operator, sigma_o = 0.5,
  multiplicative inflation 1.05 read as a float (as the reference's config
  reader does).
* ``grid_letkf_case``    small grids of the same kind for the reference-order
  LETKF.
* ``latlon_letkf_case``  360 x 180 x 10 levels x 4 variables, spherical-
  harmonic random fields (spectral slope -3, truncation T90, AR(1) vertical
  correlation), 64 members; 500k obs uniform on the sphere at random
  (continuous) levels, bilinear/linear H, sigma_o = 1; Gaspari-Cohn support
  500 km horizontally and 2 levels vertically.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

BASE_SEED = 20261203


def rng(case: int, stream: int = 0) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(BASE_SEED + 100 * case + stream))


def float_config(x: float) -> float:
    """A config number as the reference reads it: rounded to float, widened."""
    return float(np.float32(x))


# ---------------------------------------------------------------- grids ----
def _se_sqrt(n: int, length: float) -> np.ndarray:
    """Symmetric square root of the 1-D squared-exponential correlation."""
    x = np.arange(n, dtype=np.float64)
    C = np.exp(-0.5 * ((x[:, None] - x[None, :]) / length) ** 2)
    w, U = np.linalg.eigh(C)
    return (U * np.sqrt(np.clip(w, 0.0, None))) @ U.T


def grf_2d(nx: int, ny: int, length: float, sigma: float, count: int, g: np.random.Generator) -> np.ndarray:
    """`count` draws of a separable squared-exponential GRF, row-major y*nx+x."""
    Sx, Sy = _se_sqrt(nx, length), _se_sqrt(ny, length)
    Z = g.standard_normal((count, ny, nx))
    F = sigma * np.einsum("ab,kbc,dc->kad", Sy, Z, Sx)
    return F.reshape(count, ny * nx)


@dataclass
class GridCase:
    nx: int
    ny: int
    truth: np.ndarray      # n
    X: np.ndarray          # k x n members (member-major)
    obs_xy: np.ndarray     # p x 2 int32 (x, y)
    yo: np.ndarray         # p
    sigma_o: float         # float-rounded obs error
    rho: float             # float-rounded inflation
    radius: float = 0.0    # float-rounded localisation radius (grid units)

    @property
    def rvar(self) -> np.ndarray:
        return np.full(self.yo.shape[0], self.sigma_o * self.sigma_o)


def global_etkf_grid(nx: int = 64, ny: int = 64, k: int = 32, p: int = 1024, length: float = 8.0,
                     sigma_o: float = 0.5, rho: float = 1.05, case: int = 1) -> GridCase:
    g = rng(case, 0)
    fields = grf_2d(nx, ny, length, 1.0, k + 1, g)
    truth = fields[0]
    X = truth[None, :] + fields[1:]
    cells = rng(case, 1).choice(nx * ny, size=p, replace=False)
    obs_xy = np.stack([cells % nx, cells // nx], axis=1).astype(np.int32)
    so = float_config(sigma_o)
    yo = truth[cells] + so * rng(case, 2).standard_normal(p)
    return GridCase(nx, ny, truth, np.ascontiguousarray(X), obs_xy, yo, so, float_config(rho))


def grid_letkf_case(nx: int, ny: int, k: int, p: int, radius: float, rho: float = 1.05, case: int = 11,
                    length: float = 4.0, sigma_o: float = 0.5) -> GridCase:
    c = global_etkf_grid(nx, ny, k, p, length, sigma_o, rho, case)
    c.radius = float_config(radius)
    return c


# ------------------------------------------------------- lat-lon grids ----
def _legendre_table(x: np.ndarray, T: int) -> list[np.ndarray]:
    """Orthonormal associated Legendre functions; entry m is (len(x), T+1-m)."""
    nx = x.shape[0]
    s = np.sqrt(np.clip(1.0 - x * x, 0.0, None))
    out = []
    pmm = np.full(nx, np.sqrt(1.0 / (4.0 * np.pi)))
    for m in range(T + 1):
        if m > 0:
            pmm = pmm * np.sqrt((2.0 * m + 1.0) / (2.0 * m)) * s
        P = np.empty((nx, T + 1 - m))
        P[:, 0] = pmm
        if m < T:
            P[:, 1] = np.sqrt(2.0 * m + 3.0) * x * pmm
        for l in range(m + 2, T + 1):
            a = np.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
            b = np.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
            P[:, l - m] = a * (x * P[:, l - 1 - m] - b * P[:, l - 2 - m])
        out.append(P)
    return out


def sh_random_fields(count: int, nlat: int, nlon: int, T: int, slope: float, g: np.random.Generator,
                     chunk: int = 256) -> np.ndarray:
    """`count` unit-variance isotropic random fields on the cell-centred grid
    (lat_j = -90 + (j+0.5) 180/nlat, lon_i = (i+0.5) 360/nlon) with angular
    power C_l ~ l**slope for 1 <= l <= T.  Returns (count, nlat, nlon) float64."""
    lat = -90.0 + (np.arange(nlat) + 0.5) * 180.0 / nlat
    x = np.sin(np.deg2rad(lat))
    P = _legendre_table(x, T)
    ell = np.arange(T + 1, dtype=np.float64)
    Cl = np.zeros(T + 1)
    Cl[1:] = ell[1:] ** slope
    Cl *= 1.0 / np.sum((2.0 * ell + 1.0) / (4.0 * np.pi) * Cl)  # unit point variance
    sd = np.sqrt(Cl)
    lam0 = np.deg2rad(0.5 * 360.0 / nlon)
    out = np.empty((count, nlat, nlon))
    for c0 in range(0, count, chunk):
        c1 = min(count, c0 + chunk)
        nc = c1 - c0
        S = np.zeros((nc, nlat, nlon // 2 + 1), dtype=np.complex128)
        for m in range(T + 1):
            L = T + 1 - m
            re = g.standard_normal((L, nc)) * sd[m:, None]
            if m == 0:
                Fm = P[0] @ re
                S[:, :, 0] = nlon * Fm.T
            else:
                im = g.standard_normal((L, nc)) * sd[m:, None]
                Fm = P[m] @ (re - 1j * im)
                S[:, :, m] = nlon * np.sqrt(2.0) * 0.5 * Fm.T * np.exp(1j * m * lam0)
        out[c0:c1] = np.fft.irfft(S, n=nlon, axis=-1)
    return out


@dataclass
class LatLonCase:
    nlon: int
    nlat: int
    nlev: int
    nvar: int
    truth: np.ndarray        # n
    X: np.ndarray            # k x n
    obs_lat: np.ndarray
    obs_lon: np.ndarray
    obs_lev: np.ndarray
    obs_var: np.ndarray      # int32
    yo: np.ndarray
    sigma_o: float
    hsupport_km: float
    vsupport: float
    rho: float
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.nvar * self.nlev * self.nlat * self.nlon

    @property
    def rvar(self) -> np.ndarray:
        return np.full(self.yo.shape[0], self.sigma_o * self.sigma_o)

    def col_lat_lon(self) -> tuple[np.ndarray, np.ndarray]:
        lat = -90.0 + (np.arange(self.nlat) + 0.5) * 180.0 / self.nlat
        lon = (np.arange(self.nlon) + 0.5) * 360.0 / self.nlon
        la, lo = np.meshgrid(lat, lon, indexing="ij")
        return la.reshape(-1).copy(), lo.reshape(-1).copy()

    def col_base(self) -> np.ndarray:
        return np.arange(self.nlat * self.nlon, dtype=np.int64)

    @property
    def lev_stride(self) -> int:
        return self.nlat * self.nlon

    @property
    def var_stride(self) -> int:
        return self.nlev * self.nlat * self.nlon


def _vertical_ar1(F: np.ndarray, alpha: float) -> np.ndarray:
    """F: (..., nlev, nlat, nlon) independent levels -> AR(1) correlated."""
    out = np.empty_like(F)
    out[..., 0, :, :] = F[..., 0, :, :]
    s = np.sqrt(1.0 - alpha * alpha)
    for l in range(1, F.shape[-3]):
        out[..., l, :, :] = alpha * out[..., l - 1, :, :] + s * F[..., l, :, :]
    return out


def trilinear_h(field: np.ndarray, nlon, nlat, nlev, lat, lon, lev, var) -> np.ndarray:
    """The lat-lon operator (same arithmetic as the library's) on one state."""
    dlon, dlat = 360.0 / nlon, 180.0 / nlat
    gx = lon / dlon - 0.5
    fxl = np.floor(gx)
    fx = gx - fxl
    i0 = np.mod(fxl.astype(np.int64), nlon)
    i1 = (i0 + 1) % nlon
    gy = np.clip((lat + 90.0) / dlat - 0.5, 0.0, nlat - 1.0)
    j0 = np.minimum(np.floor(gy).astype(np.int64), nlat - 2)
    fy = gy - j0
    gz = np.clip(lev, 0.0, nlev - 1.0)
    l0 = np.clip(np.minimum(np.floor(gz).astype(np.int64), nlev - 2), 0, None)
    fz = gz - l0 if nlev > 1 else np.zeros_like(gz)
    l1 = l0 + 1 if nlev > 1 else l0
    plane = nlat * nlon
    vb = var.astype(np.int64) * nlev * plane

    def at(l, j, i):
        return field[vb + l * plane + j * nlon + i]

    ax, ay, az = 1.0 - fx, 1.0 - fy, 1.0 - fz
    b0 = (at(l0, j0, i0) * ax + at(l0, j0, i1) * fx) * ay + (at(l0, j0 + 1, i0) * ax + at(l0, j0 + 1, i1) * fx) * fy
    b1 = (at(l1, j0, i0) * ax + at(l1, j0, i1) * fx) * ay + (at(l1, j0 + 1, i0) * ax + at(l1, j0 + 1, i1) * fx) * fy
    return b0 * az + b1 * fz


def latlon_letkf_case(nlon: int = 360, nlat: int = 180, nlev: int = 10, nvar: int = 4, k: int = 64,
                      p: int = 500_000, T: int = 90, slope: float = -3.0, sigma_o: float = 1.0,
                      hsupport_km: float = 500.0, vsupport: float = 2.0, rho: float = 1.05,
                      alpha_v: float = 0.7, case: int = 2, clustered: float = 0.0, n_patches: int = 20,
                      patch_km: float = 800.0) -> LatLonCase:
    """Lat-lon LETKF configuration: spherical-harmonic fields (slope, T),
    AR(1) vertical correlation, p point obs at random levels and variables.
    A fraction `clustered` of the obs lies in n_patches seeded Gaussian
    patches (standard deviation patch_km), the rest uniform on the sphere."""
    g = rng(case, 0)
    nfield = (k + 1) * nvar * nlev
    F = sh_random_fields(nfield, nlat, nlon, T, slope, g)
    F = F.reshape(k + 1, nvar, nlev, nlat, nlon)
    F = _vertical_ar1(F, alpha_v)
    truth = F[0].reshape(-1).copy()
    X = (F[0][None] + F[1:]).reshape(k, -1)
    g2 = rng(case, 1)
    obs_lat = np.rad2deg(np.arcsin(g2.uniform(-1.0, 1.0, p)))
    obs_lon = g2.uniform(0.0, 360.0, p)
    if clustered > 0.0:
        gc = rng(case, 3)
        nc = int(round(clustered * p))
        clat = np.rad2deg(np.arcsin(gc.uniform(-0.9, 0.9, n_patches)))
        clon = gc.uniform(0.0, 360.0, n_patches)
        which = gc.integers(0, n_patches, nc)
        s_deg = np.rad2deg(patch_km / 6371.0)
        lat = clat[which] + s_deg * gc.standard_normal(nc)
        lon = clon[which] + s_deg * gc.standard_normal(nc) / np.cos(np.deg2rad(clat[which]))
        obs_lat[:nc] = np.clip(lat, -89.9, 89.9)
        obs_lon[:nc] = np.mod(lon, 360.0)
    obs_lev = g2.uniform(0.0, nlev - 1.0, p)
    obs_var = g2.integers(0, nvar, p).astype(np.int32)
    so = float_config(sigma_o)
    yo = trilinear_h(truth, nlon, nlat, nlev, obs_lat, obs_lon, obs_lev, obs_var) + so * rng(case, 2).standard_normal(p)
    return LatLonCase(nlon, nlat, nlev, nvar, truth, np.ascontiguousarray(X), obs_lat, obs_lon, obs_lev, obs_var,
                      yo, so, hsupport_km, vsupport, float_config(rho),
                      meta={"T": T, "slope": slope, "alpha_v": alpha_v, "case": case, "clustered": clustered})


def write_simple_state(path, values: np.ndarray, nx: int, ny: int) -> None:
    """SimpleState text format (whitespace-separated rows), full precision."""
    with open(path, "w") as f:
        for y in range(ny):
            f.write(" ".join(f"{v:.17g}" for v in values[y * nx:(y + 1) * nx]) + "\n")


def write_grid_obs(path, obs_xy: np.ndarray, yo: np.ndarray) -> None:
    """GridObservation text format (header, separator, Time Z Y X ZNU XLONG_U XLAT_U Value)."""
    with open(path, "w") as f:
        f.write("-" * 80 + "\n")
        f.write("Time Z   Y   X   ZNU      XLONG_U    XLAT_U     Simple\n")
        f.write("-" * 80 + "\n")
        for (x, y), v in zip(obs_xy, yo):
            f.write(f"0 1 {int(y)} {int(x)} 0.5 0.0 0.0 {v:.17g}\n")


@dataclass
class UnevenCase:
    X: np.ndarray        # k x n (float32-representable values, stored float64)
    obs_node: np.ndarray  # p int64 state indices (identity interpolation)
    yo: np.ndarray
    sigma_o: float
    rho: float


def uneven_batch(ncases: int = 512, n_range=(1_000, 200_000), k_choices=(20, 32, 48, 64, 100),
                 p_range=(100, 50_000), sigma_o: float = 1.0, rho: float = 1.05, case: int = 5):
    """The uneven-batch configuration: state sizes and obs counts log-uniform
    in the given ranges, member counts uniform in k_choices, obs at seeded
    state nodes (identity interpolation), sigma_o = 1.  Values are FP32
    (rounded) stored as float64.  Returns a list of UnevenCase."""
    g = rng(case, 0)
    out = []
    so = float_config(sigma_o)
    for _ in range(ncases):
        n = int(np.exp(g.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        k = int(g.choice(k_choices))
        p = int(np.exp(g.uniform(np.log(p_range[0]), np.log(p_range[1]))))
        truth = g.standard_normal(n).astype(np.float32)
        X = (truth[None, :] + g.standard_normal((k, n)).astype(np.float32)).astype(np.float64)
        nodes = g.choice(n, size=p, replace=p > n).astype(np.int64)
        yo = truth[nodes].astype(np.float64) + so * g.standard_normal(p)
        out.append(UnevenCase(X, nodes, yo, so, float_config(rho)))
    return out


# --------------------------------------------------- column operator case ----
@dataclass
class ColumnOperator:
    w: np.ndarray    # nch x nlev float32
    tau: np.ndarray  # nch float32
    nlev: int
    nch: int


def column_operator(nlev: int = 30, nch: int = 16, case: int = 4) -> ColumnOperator:
    """Seeded weights w[c,l] ~ U(0, 1)/nlev and absorption tau_c log-uniform
    in [1, 100] of the 16-channel, 30-level column operator."""
    g = rng(case, 0)
    w = (g.uniform(0.0, 1.0, (nch, nlev)) / nlev).astype(np.float32)
    tau = np.exp(g.uniform(np.log(1.0), np.log(100.0), nch)).astype(np.float32)
    return ColumnOperator(w, tau, nlev, nch)


def random_columns(ncol: int, nlev: int = 30, case: int = 4, stream: int = 1):
    """Independent levels: T ~ U(200, 310) K, q log-uniform in [1e-6, 2e-2]."""
    g = rng(case, stream)
    T = g.uniform(200.0, 310.0, (ncol, nlev)).astype(np.float32)
    q = np.exp(g.uniform(np.log(1e-6), np.log(2e-2), (ncol, nlev))).astype(np.float32)
    return T, q


@dataclass
class ColumnLetkfCase:
    nlon: int
    nlat: int
    nlev: int
    op: ColumnOperator
    truth: np.ndarray      # n = 2 nlev ncol: ((v*nlev + l)*ncol + col), v = 0 T (K), v = 1 ln q
    X: np.ndarray          # k x n
    obs_col: np.ndarray    # p int64
    obs_ch: np.ndarray     # p int32
    yo: np.ndarray         # p
    sigma_o: float
    hsupport_km: float
    rho: float

    @property
    def ncol(self) -> int:
        return self.nlat * self.nlon

    def col_lat_lon(self):
        lat = -90.0 + (np.arange(self.nlat) + 0.5) * 180.0 / self.nlat
        lon = (np.arange(self.nlon) + 0.5) * 360.0 / self.nlon
        la, lo = np.meshgrid(lat, lon, indexing="ij")
        return la.reshape(-1).copy(), lo.reshape(-1).copy()


def column_state_to_Tq(x: np.ndarray, nlev: int, ncol: int):
    """(T, ln q) state vector -> T, q columns (ncol x nlev float32)."""
    T = x[: nlev * ncol].reshape(nlev, ncol).T
    q = np.exp(x[nlev * ncol:].reshape(nlev, ncol).T)
    return np.ascontiguousarray(T, dtype=np.float32), np.ascontiguousarray(q, dtype=np.float32)


def column_letkf_case(nlon: int = 720, nlat: int = 360, nlev: int = 30, k: int = 64, p: int = 200_000,
                      T_trunc: int = 60, sigma_o: float = 0.05, hsupport_km: float = 800.0, rho: float = 1.05,
                      case: int = 4) -> ColumnLetkfCase:
    """Column grid of the learned-operator configuration: (T, ln q) columns of
    nlev levels on an nlon x nlat grid; truth and members from spherical-
    harmonic fields (T: 255 K +- 15 K; ln q: ln 2e-3 +- 1), clipped to the
    operator's ranges.  The background mean is the truth plus one error field
    (T 2 K, ln q 0.25) and the members add centred draws of the same size, so
    the spread matches the mean's actual error.  p column obs of seeded
    channels at seeded columns, y = H(truth) + N(0, sigma_o^2)."""
    op = column_operator(nlev, 16, case)
    g = rng(case, 10)
    F = sh_random_fields((k + 2) * 2 * nlev, nlat, nlon, T_trunc, -3.0, g).reshape(k + 2, 2, nlev, nlat * nlon)
    F = _vertical_ar1(F.reshape(k + 2, 2, nlev, nlat, nlon), 0.8).reshape(k + 2, 2, nlev, nlat * nlon)
    Tt = np.clip(255.0 + 15.0 * F[0, 0], 205.0, 305.0)
    lqt = np.clip(np.log(2e-3) + 1.0 * F[0, 1], np.log(2e-6), np.log(1.5e-2))
    truth = np.concatenate([Tt.reshape(-1), lqt.reshape(-1)])
    P = F[2:] - F[2:].mean(axis=0, keepdims=True)
    Tm = np.clip(Tt[None] + 2.0 * (F[1, 0][None] + P[:, 0]), 200.0, 310.0)
    lqm = np.clip(lqt[None] + 0.25 * (F[1, 1][None] + P[:, 1]), np.log(1e-6), np.log(2e-2))
    X = np.concatenate([Tm.reshape(k, -1), lqm.reshape(k, -1)], axis=1)
    ncol = nlat * nlon
    g2 = rng(case, 11)
    obs_col = g2.integers(0, ncol, p).astype(np.int64)
    obs_ch = g2.integers(0, 16, p).astype(np.int32)
    T, q = column_state_to_Tq(truth, nlev, ncol)
    y = np.zeros(p)
    cq = np.cumsum(q[obs_col].astype(np.float64), axis=1)
    Tt4 = T[obs_col].astype(np.float64) ** 4 / 1e8
    for c in range(16):
        m = obs_ch == c
        y[m] = np.sum(op.w[c].astype(np.float64) * np.exp(-float(op.tau[c]) * cq[m]) * Tt4[m], axis=1)
    so = float_config(sigma_o)
    yo = y + so * g2.standard_normal(p)
    return ColumnLetkfCase(nlon, nlat, nlev, op, truth, np.ascontiguousarray(X), obs_col, obs_ch, yo, so,
                           hsupport_km, float_config(rho))


# ------------------------------------------------ high-resolution case ----
@dataclass
class HighResCase:
    """The high-resolution LETKF configuration, generated on the GPU: members
    stored as FP32 (k x n), obs positions, levels, variables and values as
    device tensors."""
    nlon: int
    nlat: int
    nlev: int
    nvar: int
    X: "object"         # torch float32 (k, n), member-major
    truth: "object"     # torch float64 (n,)
    obs_lat: "object"
    obs_lon: "object"
    obs_lev: "object"
    obs_var: "object"   # int32
    yo: "object"
    sigma_o: float
    hsupport_km: float
    vsupport: float
    rho: float
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.nvar * self.nlev * self.nlat * self.nlon

    def col_lat_lon(self) -> tuple[np.ndarray, np.ndarray]:
        return LatLonCase.col_lat_lon(self)  # same cell-centred grid

    def col_base(self) -> np.ndarray:
        return np.arange(self.nlat * self.nlon, dtype=np.int64)

    @property
    def lev_stride(self) -> int:
        return self.nlat * self.nlon

    @property
    def var_stride(self) -> int:
        return self.nlev * self.nlat * self.nlon


def grf_fields_gpu(count: int, nlat: int, nlon: int, length_cells: float, gen, device):
    """`count` unit-variance Gaussian random fields on the nlat x nlon grid
    with squared-exponential covariance of the given length (in cells):
    white noise filtered in the 2-D Fourier domain by the square root of the
    covariance's spectrum (periodic in both directions), as float32."""
    import torch

    fy = torch.fft.fftfreq(nlat, device=device, dtype=torch.float64)
    fx = torch.fft.rfftfreq(nlon, device=device, dtype=torch.float64)
    amp = torch.exp(-(np.pi ** 2) * length_cells ** 2 * (fy[:, None] ** 2 + fx[None, :] ** 2))
    # unit variance: with orthonormal transforms the output variance is the
    # mean of |H|^2 over the full (two-sided) spectrum
    w = torch.ones_like(amp)
    w[:, 1:(nlon + 1) // 2] = 2.0  # rfft columns that stand for two frequencies
    var = float((w * amp * amp).sum() / (nlat * nlon))
    amp = (amp / np.sqrt(var)).to(torch.complex64)
    noise = torch.randn((count, nlat, nlon), generator=gen, device=device, dtype=torch.float32)
    spec = torch.fft.rfft2(noise, norm="ortho") * amp
    return torch.fft.irfft2(spec, s=(nlat, nlon), norm="ortho")


def highres_letkf_case(device, nlon: int = 1440, nlat: int = 720, nlev: int = 30, nvar: int = 4, k: int = 80,
                       p: int = 5_000_000, clustered: float = 0.6, n_patches: int = 20, patch_km: float = 800.0,
                       length_cells: float = 8.0, alpha_v: float = 0.7, sigma_o: float = 1.0,
                       hsupport_km: float = 300.0, vsupport: float = 2.0, rho: float = 0.9,
                       seed: int = 20261203 + 300) -> HighResCase:
    """High-resolution LETKF configuration: truth and members (truth plus an
    independent draw of the same field) from squared-exponential Gaussian
    random fields with AR(1) vertical correlation, members kept in FP32;
    p point obs, a fraction `clustered` in n_patches Gaussian patches
    (standard deviation patch_km), the rest uniform on the sphere, at
    uniform random levels and variables, y = H(truth) + N(0, sigma_o^2)."""
    import torch

    from . import kernels as K

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    n = nvar * nlev * nlat * nlon
    s = float(np.sqrt(1.0 - alpha_v * alpha_v))

    def draw():  # (nvar, nlev, nlat, nlon) float32, AR(1) in the vertical
        F = grf_fields_gpu(nvar * nlev, nlat, nlon, length_cells, g, device).view(nvar, nlev, nlat, nlon)
        for l in range(1, nlev):
            F[:, l] = alpha_v * F[:, l - 1] + s * F[:, l]
        return F.reshape(-1)

    truth32 = draw()
    X = torch.empty((k, n), dtype=torch.float32, device=device)
    for i in range(k):
        X[i] = truth32 + draw()
    truth = truth32.double()
    # observations
    rng_ = np.random.default_rng(seed + 1)
    lat = np.rad2deg(np.arcsin(rng_.uniform(-1.0, 1.0, p)))
    lon = rng_.uniform(0.0, 360.0, p)
    nc = int(round(clustered * p))
    if nc > 0:
        clat = np.rad2deg(np.arcsin(rng_.uniform(-0.9, 0.9, n_patches)))
        clon = rng_.uniform(0.0, 360.0, n_patches)
        which = rng_.integers(0, n_patches, nc)
        s_deg = np.rad2deg(patch_km / 6371.0)
        lat[:nc] = np.clip(clat[which] + s_deg * rng_.standard_normal(nc), -89.9, 89.9)
        lon[:nc] = np.mod(clon[which] + s_deg * rng_.standard_normal(nc) / np.cos(np.deg2rad(clat[which])), 360.0)
    lev = rng_.uniform(0.0, nlev - 1.0, p)
    var = rng_.integers(0, nvar, p).astype(np.int32)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)  # noqa: E731
    olat, olon, olev, ovar = T(lat), T(lon), T(lev), T(var)
    so = float_config(sigma_o)
    hx_truth = K.hx_latlon(truth[None, :].contiguous(), nlon, nlat, nlev, olat, olon, olev, ovar)[:, 0]
    yo = hx_truth + so * T(rng_.standard_normal(p))
    return HighResCase(nlon, nlat, nlev, nvar, X, truth, olat, olon, olev, ovar, yo, so, hsupport_km, vsupport,
                       float_config(rho), meta={"length_cells": length_cells, "alpha_v": alpha_v,
                                                "clustered": clustered, "n_patches": n_patches,
                                                "patch_km": patch_km, "seed": seed})
