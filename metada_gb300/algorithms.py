"""Python mirror of METADA's analysis-algorithm policy over the GPU library.

The reference selects ``ETKF<Tag>`` / ``LETKF<Tag>`` with the signature
``(Ensemble&, Observation&, const ObsOperator&, const Config&)`` and calls
``Analyse()`` then ``saveEnsemble()`` (src/framework/algorithms/ETKF.hpp:86-200,
LETKF.hpp:47-142).  These classes keep that surface: the same constructor
arguments and config keys (``inflation``, ``localization_radius``,
``output_base_file``, ``format``; numbers rounded to float as the reference's
config reader does, ConfigValue.hpp:108), the same method names, and the same
error behaviour (exceptions on bad input).  Data live in GPU memory; host
arrays are copied in once and read back lazily.

Extra config keys select the GB300 paths: ``precision`` ("fp64" | "mixed"),
``semantics`` ("reference" | "hunt"), ``order`` ("sequential" | "batched",
LETKF), ``vertical_radius`` (levels) and ``rtps`` (relaxation alpha).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import torch

from . import _lib
from . import kernels as K
from .synthetic import float_config


def _cfg_float(config: dict, key: str, default=None) -> float:
    if key not in config:
        if default is None:
            raise KeyError(f"missing config key '{key}'")
        return float(default)
    return float_config(config[key])


class SimpleGeometry:
    """2-D grid, row-major y*x_dim + x (SimpleGeometry.hpp:42-55)."""

    def __init__(self, x_dim: int, y_dim: int):
        if x_dim <= 0 or y_dim <= 0:
            raise ValueError("SimpleGeometry: x_dim and y_dim must be positive")
        self.x_dim, self.y_dim = int(x_dim), int(y_dim)

    def size(self) -> int:
        return self.x_dim * self.y_dim


class LatLonGeometry:
    """Cell-centred lat-lon grid with levels and variables, layout
    ((v*nlev + l)*nlat + j)*nlon + i."""

    def __init__(self, nlon: int, nlat: int, nlev: int = 1, nvar: int = 1):
        self.nlon, self.nlat, self.nlev, self.nvar = int(nlon), int(nlat), int(nlev), int(nvar)

    def size(self) -> int:
        return self.nvar * self.nlev * self.nlat * self.nlon

    def columns(self) -> tuple[np.ndarray, np.ndarray]:
        lat = -90.0 + (np.arange(self.nlat) + 0.5) * 180.0 / self.nlat
        lon = (np.arange(self.nlon) + 0.5) * 360.0 / self.nlon
        la, lo = np.meshgrid(lat, lon, indexing="ij")
        return la.reshape(-1).copy(), lo.reshape(-1).copy()


class Ensemble:
    """k members on the device (member-major), as Ensemble.hpp:40-195 holds them."""

    def __init__(self, members, geometry, device: str | torch.device = "cuda:0"):
        self.geometry = geometry
        self.device = torch.device(device)
        if isinstance(members, torch.Tensor):
            X = members.to(self.device, dtype=torch.float64)
        else:
            X = torch.as_tensor(np.ascontiguousarray(members, dtype=np.float64))
            if X.device.type == "cpu" and self.device.type == "cuda":
                X = X.pin_memory() if not X.is_pinned() else X
            X = X.to(self.device, non_blocking=True)
        if X.dim() != 2 or X.shape[1] != geometry.size():
            raise ValueError(f"Ensemble: members must be k x {geometry.size()}")
        self.X = X.contiguous()
        self._mean: torch.Tensor | None = None

    def Size(self) -> int:
        return int(self.X.shape[0])

    def GetMember(self, index: int) -> np.ndarray:
        if not 0 <= index < self.Size():
            raise IndexError("Ensemble member index out of range")
        return self.X[index].cpu().numpy()

    def RecomputeMean(self) -> None:
        self._mean = K.ens_mean(self.X)

    def Mean(self) -> np.ndarray:
        return self.mean_tensor().cpu().numpy()

    def mean_tensor(self) -> torch.Tensor:
        """Ensemble::Mean() on the device (computed once, then cached)."""
        if self._mean is None:
            self.RecomputeMean()
        return self._mean

    def RecomputePerturbations(self) -> torch.Tensor:
        self._mean, Xp = K.ens_mean_pert(self.X)
        return Xp

    def to_host(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            return self.X.cpu().numpy()
        torch.from_numpy(out).copy_(self.X)
        return out


class Observation:
    """Point observations: values, error standard deviations, locations
    (GridObservation.hpp / PointObservation.hpp).  ``grid_xy`` (p x 2 ints)
    for grid coordinates, or ``lat``/``lon``/``lev``/``var`` for geographic."""

    def __init__(self, values, error, *, grid_xy=None, lat=None, lon=None, lev=None, var=None, valid=None,
                 device: str | torch.device = "cuda:0"):
        dev = torch.device(device)
        values = np.ascontiguousarray(values, dtype=np.float64)
        p = values.shape[0]
        err = np.broadcast_to(np.asarray(error, dtype=np.float64), (p,))
        self.valid = None if valid is None else np.ascontiguousarray(valid, dtype=np.uint8)
        rvar = err * err
        if self.valid is not None:
            rvar = np.where(self.valid != 0, rvar, np.inf)  # GridObservation.hpp:243-249
        self._host = {"values": values, "rvar": rvar}

        def d(a, dt):
            return None if a is None else torch.as_tensor(np.ascontiguousarray(a, dtype=dt)).to(dev)

        self.yo = d(values, np.float64)
        self.rvar = d(rvar, np.float64)
        self.grid_xy = d(grid_xy, np.int32)
        self.lat, self.lon, self.lev = d(lat, np.float64), d(lon, np.float64), d(lev, np.float64)
        self.var = d(var, np.int32)
        self.valid_d = d(self.valid, np.uint8)
        if self.grid_xy is None and self.lat is None:
            raise ValueError("Observation: give grid_xy or lat/lon")

    def size(self) -> int:
        return int(self.yo.shape[0])

    def getObservationValues(self) -> np.ndarray:
        return self._host["values"].copy()

    def getCovariance(self) -> np.ndarray:
        return self._host["rvar"].copy()


class ObsOperator:
    """H: IDW4 for grid observations on a SimpleGeometry
    (IdentityObsOperator.hpp:154-180), bilinear/linear on a LatLonGeometry."""

    def apply(self, ensemble: Ensemble, obs: Observation) -> torch.Tensor:
        g = ensemble.geometry
        if isinstance(g, SimpleGeometry):
            if obs.grid_xy is None:
                raise ValueError("IDW4 operator needs grid observations")
            return K.hx_idw4(ensemble.X, g.x_dim, g.y_dim, obs.grid_xy, obs.valid_d)
        if obs.lat is None:
            raise ValueError("lat-lon operator needs geographic observations")
        var = obs.var if obs.var is not None else torch.zeros_like(obs.yo, dtype=torch.int32)
        lev = obs.lev if obs.lev is not None else torch.zeros_like(obs.yo)
        return K.hx_latlon(ensemble.X, g.nlon, g.nlat, g.nlev, obs.lat, obs.lon, lev, var)


def _precision(config: dict) -> int:
    p = str(config.get("precision", "fp64")).lower()
    if p not in ("fp64", "mixed"):
        raise ValueError("precision must be 'fp64' or 'mixed'")
    return _lib.MG_PREC_FP64 if p == "fp64" else _lib.MG_PREC_MIXED


def _flags(config: dict) -> int:
    sem = str(config.get("semantics", "reference")).lower()
    if sem == "reference":
        return _lib.MG_COMPAT
    if sem != "hunt":
        raise ValueError("semantics must be 'reference' or 'hunt'")
    return _lib.MG_RTPS if "rtps" in config else 0


def _save_state(path: Path, values: torch.Tensor, geometry) -> None:
    """One state of the ensemble (a float64 device vector) to a file: for a
    SimpleGeometry the text of SimpleState::saveToFile ("%12.6f" rows,
    SimpleState.hpp:160-188), formatted on the device; otherwise the exact
    values as a binary .npy."""
    path.parent.mkdir(parents=True, exist_ok=True)
    if isinstance(geometry, SimpleGeometry):
        path.write_bytes(K.format_state(values, geometry.x_dim, geometry.y_dim))
    else:
        np.save(path.with_suffix(".npy"), values.cpu().numpy())


class ETKF:
    """Global ETKF (ETKF.hpp:76-210)."""

    def __init__(self, ensemble: Ensemble, obs: Observation, obs_op: ObsOperator, config: dict):
        self.ensemble, self.obs, self.obs_op = ensemble, obs, obs_op
        self.inflation = _cfg_float(config, "inflation")
        self.output_base_file = str(config.get("output_base_file", "analysis"))
        self.format = str(config.get("format", "txt"))
        self.precision = _precision(config)
        self.flags = _flags(config)
        self._saved_mean: torch.Tensor | None = None

    def Analyse(self) -> None:
        HX = self.obs_op.apply(self.ensemble, self.obs)
        self._saved_mean = K.etkf(self.ensemble.X, HX, self.obs.yo, self.obs.rvar, self.inflation, flags=self.flags,
                                  precision=self.precision)
        # The reference leaves the background mean in Ensemble::Mean() (ETKF.hpp:190-191).
        self.ensemble._mean = self._saved_mean

    def saveEnsemble(self) -> None:
        base = Path(self.output_base_file)
        _save_state(Path(f"{base}_mean.{self.format}"), self.ensemble.mean_tensor(), self.ensemble.geometry)
        for i in range(self.ensemble.Size()):
            _save_state(Path(f"{base}_member_{i}.{self.format}"), self.ensemble.X[i], self.ensemble.geometry)


class EnKF:
    """Stochastic EnKF with perturbed observations (EnKF.hpp:99-254).  The
    reference draws the perturbations eps = chol_L(R) z, z ~ N(0, 1), from
    an unseeded std::mt19937 (:336-352); here z comes from a seeded numpy
    generator (config key ``seed``, default 0), obs-major like the
    reference's loop, so analyses are reproducible.  ``inflation_method``
    is read as the reference reads it; every method scales the perturbations
    by sqrt(inflation) (:322-335)."""

    def __init__(self, ensemble: Ensemble, obs: Observation, obs_op: ObsOperator, config: dict):
        self.ensemble, self.obs, self.obs_op = ensemble, obs, obs_op
        self.inflation = _cfg_float(config, "inflation")
        method = str(config.get("inflation_method", "multiplicative"))
        self.inflation_method = method if method in ("multiplicative", "additive", "relaxation") else "multiplicative"
        self.output_base_file = str(config.get("output_base_file", "analysis"))
        self.format = str(config.get("format", "txt"))
        self.precision = _precision(config)
        self.seed = int(config.get("seed", 0))
        self.results: dict = {}

    def Analyse(self) -> None:
        HX = self.obs_op.apply(self.ensemble, self.obs)
        k = self.ensemble.Size()
        p = self.obs.size()
        z = np.random.default_rng(self.seed).standard_normal((p, k))
        cov = self.obs.getCovariance()
        sigma = np.sqrt(np.where(np.isfinite(cov), cov, 0.0))  # invalid obs (R = +inf) carry no weight
        eps = torch.as_tensor(sigma[:, None] * z, device=self.ensemble.X.device)
        mean, diag = K.enkf(self.ensemble.X, HX, self.obs.yo, self.obs.rvar, eps, self.inflation,
                            precision=self.precision)
        self.ensemble._mean = mean
        self.results = {**diag, "ensemble_size": k, "observation_count": p,
                        "inflation_method": self.inflation_method, "inflation_factor": self.inflation}

    def getAnalysisResults(self) -> dict:
        return dict(self.results)

    def saveEnsemble(self) -> None:
        base = Path(self.output_base_file)
        _save_state(Path(f"{base}_mean.{self.format}"), self.ensemble.mean_tensor(), self.ensemble.geometry)
        for i in range(self.ensemble.Size()):
            _save_state(Path(f"{base}_member_{i}.{self.format}"), self.ensemble.X[i], self.ensemble.geometry)


class LETKF:
    """Local ETKF (LETKF.hpp:37-253).  ``order = "sequential"`` reproduces the
    reference's in-place, grid-point-ordered analysis on a SimpleGeometry;
    ``order = "batched"`` runs all local analyses at once with the background
    obs-space prior (the GB300 path)."""

    def __init__(self, ensemble: Ensemble, obs: Observation, obs_op: ObsOperator, config: dict):
        self.ensemble, self.obs, self.obs_op = ensemble, obs, obs_op
        self.inflation = _cfg_float(config, "inflation")
        self.localization_radius = _cfg_float(config, "localization_radius")
        self.vertical_radius = _cfg_float(config, "vertical_radius", 0.0)
        self.output_base_file = str(config.get("output_base_file", "analysis"))
        self.format = str(config.get("format", "nc"))
        self.precision = _precision(config)
        self.flags = _flags(config)
        self.order = str(config.get("order", "batched"))
        if "rtps" in config:
            self.inflation = _cfg_float(config, "rtps")
        self.stats = None
        self._lists = None

    def _local_lists(self):
        g = self.ensemble.geometry
        if isinstance(g, SimpleGeometry):
            off, idx = K.select_grid(g.x_dim, g.y_dim, self.obs.grid_xy, self.localization_radius)
            return off, idx, None
        la, lo = g.columns()
        dev = self.ensemble.X.device
        return K.select_geo(torch.from_numpy(la).to(dev), torch.from_numpy(lo).to(dev), self.obs.lat, self.obs.lon,
                            self.localization_radius)

    def Analyse(self) -> None:
        g = self.ensemble.geometry
        if self.order == "sequential":
            if not isinstance(g, SimpleGeometry) or self.flags != _lib.MG_COMPAT or self.precision != _lib.MG_PREC_FP64:
                raise ValueError("sequential order is the reference LETKF: SimpleGeometry, reference semantics, fp64")
            self.ensemble._mean = K.letkf_compat_grid(self.ensemble.X, g.x_dim, g.y_dim, self.obs.grid_xy,
                                                      self.obs.yo, self.localization_radius, self.inflation,
                                                      self.obs.valid_d)
            return
        HX = self.obs_op.apply(self.ensemble, self.obs)
        off, idx, dist = self._local_lists()
        dev = self.ensemble.X.device
        if isinstance(g, SimpleGeometry):
            col_base = torch.arange(g.size(), dtype=torch.int64, device=dev)
            kw = dict(nlev=1, n_var=1, lev_stride=0, var_stride=0)
        else:
            col_base = torch.arange(g.nlat * g.nlon, dtype=torch.int64, device=dev)
            kw = dict(nlev=g.nlev, n_var=g.nvar, lev_stride=g.nlat * g.nlon, var_stride=g.nlev * g.nlat * g.nlon,
                      obs_lev=self.obs.lev if g.nlev > 1 else None)
        self.ensemble._mean, self.stats = K.letkf_batched(
            self.ensemble.X, col_base=col_base, HX=HX, yo=self.obs.yo, rvar=self.obs.rvar, loc_off=off,
            loc_idx=idx, loc_dist=dist, hsupport=self.localization_radius, vsupport=self.vertical_radius,
            rho=self.inflation, flags=self.flags, precision=self.precision, **kw)

    def saveEnsemble(self) -> None:
        base = Path(self.output_base_file)
        _save_state(Path(f"{base}_mean.{self.format}"), self.ensemble.mean_tensor(), self.ensemble.geometry)
        for i in range(self.ensemble.Size()):
            _save_state(Path(f"{base}_member_{i}.{self.format}"), self.ensemble.X[i], self.ensemble.geometry)


class Metrics:
    """Ensemble diagnostics, the reference's Metrics<double>
    (src/framework/algorithms/Metrics.hpp:74-94), computed on the device."""

    @staticmethod
    def CalculateAll(ensemble, truth, state_dim: int | None = None, ens_size: int | None = None) -> dict:
        """ensemble: an Ensemble, or members as a k x n array; truth: n values.
        Returns mean, spread (numpy), rmse, bias, correlation, crps,
        avg_spread."""
        if isinstance(ensemble, Ensemble):
            X = ensemble.X
            dev = X.device
        else:
            dev = torch.device("cuda", torch.cuda.current_device())
            X = torch.as_tensor(np.asarray(ensemble, dtype=np.float64), device=dev)
        if state_dim is not None and state_dim != X.shape[1]:
            raise ValueError("state_dim does not match the members")
        if ens_size is not None and ens_size != X.shape[0]:
            raise ValueError("ens_size does not match the members")
        t = torch.as_tensor(np.asarray(truth, dtype=np.float64), device=dev)
        mean, spread, vals = K.ens_metrics(X.contiguous(), t)
        return {"mean": mean.cpu().numpy(), "spread": spread.cpu().numpy(), **vals}
