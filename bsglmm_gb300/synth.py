"""Seeded synthetic studies with the shapes of the sampler's benchmark
configurations.

There is no public lesion dataset for this model and the reference ships no
lesion maps or design file, so studies are generated: coefficient fields are
Gaussian-smoothed white noise standardised within the mask, the design has
an intercept, a +-0.5 group column and the stated covariates, and
Y_iv ~ Bernoulli(Phi(x_i' beta_v)).

Arrays use the reference layouts: mask [Z][Y][X] (x fastest), covar [P][N],
data [N][V] by compact mask index, beta [P][V].
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
from scipy import ndimage, special


@dataclass
class Study:
    name: str
    mask: np.ndarray          # uint8 [Z][Y][X]
    covar: np.ndarray         # float32 [P][N]
    data: np.ndarray          # uint8 [N][V]
    beta_true: np.ndarray     # float32 [P][V]
    nsubtypes: int = 1
    names: list = field(default_factory=list)

    @property
    def shape(self):
        return self.mask.shape

    @property
    def N(self):
        return self.covar.shape[1]

    @property
    def P(self):
        return self.covar.shape[0]

    @property
    def V(self):
        return int(self.mask.astype(bool).sum())


def sphere_mask(n: int, radius: float, center=None) -> np.ndarray:
    """Cube of side n; voxel centres at 1-based coordinates (as the
    reference's padded grid), sphere about `center` (1-based)."""
    c = (n + 1) / 2.0 if center is None else center
    g = np.arange(1, n + 1, dtype=np.float64)
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    return (((x - c) ** 2 + (y - c) ** 2 + (z - c) ** 2) <= radius * radius).astype(np.uint8)


def ellipsoid_mask(shape_xyz, semi_axes_xyz) -> np.ndarray:
    X, Y, Z = shape_xyz
    ax, ay, az = semi_axes_xyz
    cx, cy, cz = (X + 1) / 2.0, (Y + 1) / 2.0, (Z + 1) / 2.0
    z, y, x = np.meshgrid(np.arange(1, Z + 1), np.arange(1, Y + 1),
                          np.arange(1, X + 1), indexing="ij")
    r = ((x - cx) / ax) ** 2 + ((y - cy) / ay) ** 2 + ((z - cz) / az) ** 2
    return (r <= 1.0).astype(np.uint8)


def smooth_field(rng: np.random.Generator, mask: np.ndarray, fwhm: float,
                 mean: float, sd: float) -> np.ndarray:
    """White noise smoothed with sigma = FWHM / 2.3548, standardised within
    the mask to (mean, sd); returned by compact mask index (x fastest)."""
    noise = rng.standard_normal(mask.shape)
    f = ndimage.gaussian_filter(noise, sigma=fwhm / 2.3548, mode="constant")
    v = f[mask.astype(bool)]
    v = (v - v.mean()) / (v.std() + 1e-12)
    return (mean + sd * v).astype(np.float32)


def draw_outcomes(rng: np.random.Generator, covar: np.ndarray,
                  beta: np.ndarray, chunk: int = 1 << 16) -> np.ndarray:
    """Y_iv ~ Bernoulli(Phi(x_i' beta_v)) as uint8 [N][V]."""
    P, N = covar.shape
    V = beta.shape[1]
    out = np.empty((N, V), dtype=np.uint8)
    X = covar.T.astype(np.float64)
    for v0 in range(0, V, chunk):
        eta = X @ beta[:, v0:v0 + chunk].astype(np.float64)
        p = special.ndtr(eta)
        out[:, v0:v0 + chunk] = rng.random(eta.shape) < p
    return out


def design(rng: np.random.Generator, N: int, P: int, kind: str) -> np.ndarray:
    """Design matrix [P][N].  kind "c0": intercept, group +-0.5, N(0,1);
    "brain": intercept, group, age N(0,1), sex +-0.5, lognormal(0,0.5)
    standardised, then N(0,1) nuisance columns."""
    cols = [np.ones(N), np.where(rng.random(N) < 0.5, 0.5, -0.5)]
    if kind == "brain":
        cols.append(rng.standard_normal(N))
        cols.append(np.where(rng.random(N) < 0.5, 0.5, -0.5))
        lv = rng.lognormal(0.0, 0.5, N)
        cols.append((lv - lv.mean()) / lv.std())
    while len(cols) < P:
        cols.append(rng.standard_normal(N))
    return np.stack(cols[:P]).astype(np.float32)


def make_study(name: str, mask: np.ndarray, N: int, P: int, fwhm: float,
               intercept_p: float, seed: int, kind: str = "c0") -> Study:
    rng = np.random.default_rng(seed)
    X = design(rng, N, P, kind)
    if kind == "c0":
        X = X[:P]
    b = [smooth_field(rng, mask, fwhm, special.ndtri(intercept_p), 0.5)]
    for _ in range(1, P):
        b.append(smooth_field(rng, mask, fwhm, 0.0, 0.3))
    beta = np.stack(b)
    data = draw_outcomes(rng, X, beta)
    names = ["Intercept", "Group", "Age", "Sex", "LesionVol"] + [
        f"Nuis{i}" for i in range(1, 9)]
    return Study(name, mask, X, data, beta, 1, names[:P])


# ------------------------------------------------------- the benchmark studies --
def config0(seed: int = 0) -> Study:
    """20^3 grid, sphere r = 9 about (10.5, 10.5, 10.5), N = 50, P = 3,
    FWHM 3, intercept Phi^-1(0.05)."""
    return make_study("c0", sphere_mask(20, 9.0, 10.5), 50, 3, 3.0, 0.05, seed)


BRAIN_SHAPE = (91, 109, 91)
BRAIN_AXES = (35.8, 42.9, 35.8)


def config1(seed: int = 1, N: int = 1000) -> Study:
    """91x109x91 grid, ellipsoid of about 230k voxels, N = 1000, P = 5,
    FWHM 4, intercept Phi^-1(0.03)."""
    return make_study("c1", ellipsoid_mask(BRAIN_SHAPE, BRAIN_AXES), N, 5,
                      4.0, 0.03, seed, "brain")


def config2(seed: int = 2) -> Study:
    """The brain-sized ellipsoid mask with N = 2000 and P = 8."""
    return make_study("c2", ellipsoid_mask(BRAIN_SHAPE, BRAIN_AXES), 2000, 8,
                      4.0, 0.03, seed, "brain")


def config3(seed: int = 3, ndatasets: int = 64):
    """Replicate studies: cube side U{32..64}, sphere radius 60-90% of the
    half side, N U{40..400}, P U{2..6}, the 20^3 study's recipe, per-study seeds."""
    rng = np.random.default_rng(seed)
    out = []
    for d in range(ndatasets):
        n = int(rng.integers(32, 65))
        frac = float(rng.uniform(0.6, 0.9))
        N = int(rng.integers(40, 401))
        P = int(rng.integers(2, 7))
        out.append(make_study(f"c3_{d}", sphere_mask(n, frac * n / 2.0), N, P,
                              3.0, 0.05, seed * 1000 + d))
    return out


BIG_SHAPE = (182, 218, 182)
BIG_AXES = (66.9, 80.1, 66.9)


def config4(seed: int = 4) -> Study:
    """182x218x182 grid, ellipsoid of about 1.5M voxels, N = 500, P = 6,
    intercept Phi^-1(0.02)."""
    return make_study("c4", ellipsoid_mask(BIG_SHAPE, BIG_AXES), 500, 6, 4.0,
                      0.02, seed, "brain")


def small_study(seed: int, shape=(10, 9, 8), N: int = 37, P: int = 4,
                S: int = 2, fill: float = 0.55) -> Study:
    """Irregular blob mask touching the grid faces, with an isolated voxel,
    for parity tests (ragged N, several group columns)."""
    rng = np.random.default_rng(seed)
    X, Y, Z = shape
    noise = ndimage.gaussian_filter(rng.standard_normal((Z, Y, X)), 1.0)
    mask = (noise > np.quantile(noise, 1.0 - fill)).astype(np.uint8)
    mask[0, 0, 0] = 1                      # corner voxel on the grid face
    mask[0, 0, 1] = mask[0, 1, 0] = mask[1, 0, 0] = 0  # isolate it
    cov = [np.ones(N)]
    for g in range(1, S):
        cov.append(np.where(rng.random(N) < 0.5, 0.5, -0.5))
    while len(cov) < P:
        cov.append(rng.standard_normal(N))
    covar = np.stack(cov[:P]).astype(np.float32)
    V = int(mask.sum())
    beta = np.stack([rng.normal(-1.0 if p == 0 else 0.0, 0.4, V)
                     for p in range(P)]).astype(np.float32)
    data = draw_outcomes(rng, covar, beta)
    return Study(f"small{seed}", mask, covar, data, beta, S,
                 [f"c{p}" for p in range(P)])
