"""Seeded synthetic inputs for the CA workloads.

Every generator is deterministic from its seed (splitmix64 stream) and
platform independent: real fields are quantised to multiples of 2**-10, so
an ulp of difference in ``exp`` between two machines' libm cannot change the
stored bits except at a rounding tie.

Workloads (shapes and distributions of the benchmark configurations):
  * Life B3/S23: cells alive i.i.d. Bernoulli(p), p = 0.3.
  * SCIDDICA-T: DEM = 0.3 * row index + 20 Gaussian hills (amplitude
    U[10, 200] m, sigma U[20, 200] cells, uniform centres), clipped to
    [0, 2000] m; thickness 0 except one elliptical source (semi-axes
    U[20, 80] cells, peak depth U[1, 20] m, paraboloid profile) placed at
    least ``margin`` cells from every edge, in the upper half of the rows (the
    plane falls towards row 0, so this leaves the flow the longest path).
"""
from __future__ import annotations

import numpy as np

_MASK = (1 << 64) - 1


class SplitMix64:
    """splitmix64 (Steele, Lea, Flood 2014), the generator named for the inputs."""

    def __init__(self, seed: int):
        self.state = seed & _MASK

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & _MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
        return z ^ (z >> 31)

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> float:
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / 9007199254740992.0))


def splitmix64_array(seed: int, n: int) -> np.ndarray:
    """n consecutive splitmix64 outputs (vectorised; uint64 arithmetic wraps)."""
    with np.errstate(over="ignore"):
        k = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed & _MASK) + k * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform_array(seed: int, shape) -> np.ndarray:
    n = int(np.prod(shape))
    u = (splitmix64_array(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return u.reshape(shape)


def quantise(x: np.ndarray, bits: int = 10) -> np.ndarray:
    s = float(1 << bits)
    return np.floor(x * s) / s


def life_state(rows: int, cols: int, p: float = 0.3, seed: int = 1) -> np.ndarray:
    """Bernoulli(p) alive cells as uint8 0/1, row-major (rows, cols)."""
    return (uniform_array(seed, (rows, cols)) < p).astype(np.uint8)


def life3d_state(rows: int, cols: int, slices: int, p: float = 0.1, seed: int = 7) -> np.ndarray:
    """Bernoulli(p) cells in OpenCAL's 3D layout: array shape (slices, rows, cols)."""
    return (uniform_array(seed, (slices, rows, cols)) < p).astype(np.uint8)


def sciddicaT_inputs(rows: int, cols: int, seed: int = 2, hills: int = 20, margin: int | None = None,
                     semi_axes=(20.0, 80.0), sigma=(20.0, 200.0)):
    """(z, h) float64 arrays of shape (rows, cols) for SCIDDICA-T.

    ``margin`` defaults to 300 cells on grids of at least 1024 cells per side
    and to rows // 4 on smaller grids; the source never comes closer to an
    edge than that.  Semi-axes and sigma shrink in proportion on grids
    smaller than 2048 cells per side so that small parity grids keep the
    same shape of problem.
    """
    rng = SplitMix64(seed)
    scale = min(1.0, min(rows, cols) / 2048.0)
    if margin is None:
        margin = 300 if min(rows, cols) >= 1024 else max(4, min(rows, cols) // 4)
    ii = np.arange(rows, dtype=np.float64)[:, None]
    jj = np.arange(cols, dtype=np.float64)[None, :]
    z = 0.3 * ii + 0.0 * jj
    for _ in range(hills):
        amp = rng.uniform(10.0, 200.0)
        sg = rng.uniform(sigma[0], sigma[1]) * scale
        ci = rng.uniform(0.0, rows - 1.0)
        cj = rng.uniform(0.0, cols - 1.0)
        z = z + amp * np.exp(-((ii - ci) ** 2 + (jj - cj) ** 2) / (2.0 * sg * sg))
    z = quantise(np.clip(z, 0.0, 2000.0))

    a = max(2.0, rng.uniform(semi_axes[0], semi_axes[1]) * scale)
    b = max(2.0, rng.uniform(semi_axes[0], semi_axes[1]) * scale)
    depth = rng.uniform(1.0, 20.0)
    lo_i, hi_i = margin + a, rows - 1 - margin - a
    lo_j, hi_j = margin + b, cols - 1 - margin - b
    # the plane falls towards row 0: start the source in the upper half so the
    # flow has the longest possible path before it could reach an edge
    ci = rng.uniform(max(lo_i, 0.55 * rows), max(lo_i, 0.55 * rows, hi_i))
    cj = rng.uniform(lo_j, max(lo_j, hi_j))
    r2 = ((ii - ci) / a) ** 2 + ((jj - cj) / b) ** 2
    h = np.where(r2 < 1.0, depth * (1.0 - r2), 0.0)
    h = quantise(h)
    return np.ascontiguousarray(z), np.ascontiguousarray(h)


def random_field(shape, seed: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
    return quantise(lo + (hi - lo) * uniform_array(seed, shape))


def sparse_blobs(shape, seed: int, n_blobs: int = 3, radius: float = 3.0, peak: float = 8.0,
                 margin: int = 4) -> np.ndarray:
    """A few quantised bumps away from the edges (2D or 3D; shape is the array shape)."""
    rng = SplitMix64(seed)
    grids = np.meshgrid(*[np.arange(s, dtype=np.float64) for s in shape], indexing="ij")
    v = np.zeros(shape, dtype=np.float64)
    for _ in range(n_blobs):
        c = [rng.uniform(margin + radius, s - 1 - margin - radius) for s in shape]
        r2 = sum((g - ci) ** 2 for g, ci in zip(grids, c)) / (radius * radius)
        v = v + np.where(r2 < 1.0, peak * (1.0 - r2), 0.0)
    return quantise(v)


def ensemble_spec(n: int, seed: int = 4, size_range=(128, 1024), p_r_range=(0.3, 0.7),
                  p_eps_range=(5e-4, 5e-3)):
    """Dimensions and parameters of a calibration ensemble of ``n`` SCIDDICA-T
    instances: rows and cols independently uniform in ``size_range``
    (inclusive), p_r and p_eps uniform in their ranges; instance i's DEM and
    source come from ``sciddicaT_inputs(rows, cols, seed=1000 + i)``.
    Returns (dims [(rows, cols)], params [(p_r, p_eps)])."""
    rng = SplitMix64(seed)
    lo, hi = size_range
    dims, params = [], []
    for _ in range(n):
        rows = lo + int(rng.next_u64() % (hi - lo + 1))
        cols = lo + int(rng.next_u64() % (hi - lo + 1))
        dims.append((rows, cols))
        params.append((rng.uniform(*p_r_range), rng.uniform(*p_eps_range)))
    return dims, params


def ensemble_inputs(dims, first_seed: int = 1000):
    """(z list, h list) for the instances of an ensemble."""
    zs, hs = [], []
    for i, (rows, cols) in enumerate(dims):
        z, h = sciddicaT_inputs(rows, cols, seed=first_seed + i)
        zs.append(z)
        hs.append(h)
    return zs, hs


# SCIARA-fv2 parameters of the reference's 2006 configuration file, in the
# file's order (Pclock, PTsol, PTvent, Pr(Tsol), Pr(Tvent), Phc(Tsol),
# Phc(Tvent), Pcool, Prho, Pepsilon, Psigma, Pcv), plus the cell size Pc.
SCIARA_PARAMS = (60.0, 1143.0, 1360.0, 0.075, 0.90, 60.0, 0.4, 9.0, 2600.0, 0.90, 5.68e-08, 1150.0, 10.0)


def _value_noise(rows: int, cols: int, seed: int, octaves: int = 5, base: int = 64) -> np.ndarray:
    """Sum of bilinearly interpolated random lattices, one per octave (lattice
    spacing halving, amplitude halving), scaled to [-1, 1]."""
    rng_seed = seed
    out = np.zeros((rows, cols))
    amp = 1.0
    step = float(base)
    total = 0.0
    for _ in range(octaves):
        gr = int(rows / step) + 2
        gc = int(cols / step) + 2
        lat = uniform_array(rng_seed, (gr, gc)) * 2.0 - 1.0
        rng_seed += 1
        y = np.arange(rows, dtype=np.float64)[:, None] / step
        x = np.arange(cols, dtype=np.float64)[None, :] / step
        y0 = np.floor(y).astype(np.int64)
        x0 = np.floor(x).astype(np.int64)
        fy = y - y0
        fx = x - x0
        v = (lat[y0, x0] * (1 - fy) * (1 - fx) + lat[y0 + 1, x0] * fy * (1 - fx) +
             lat[y0, x0 + 1] * (1 - fy) * fx + lat[y0 + 1, x0 + 1] * fy * fx)
        out = out + amp * v
        total += amp
        amp *= 0.5
        step = max(step / 2.0, 1.0)
    return out / total


def sciara_inputs(rows: int, cols: int, seed: int = 5, cell: float = 10.0, nvents: int | None = None,
                  phases: int = 6, rate_range=(10.0, 50.0), slope: float = 3000.0 / 20480.0):
    """A synthetic volcano for SCIARA-fv2: a cone (height falling linearly
    from the centre with the given slope, 3000 m over 20.48 km on a 4096^2
    grid of 10 m cells, clipped at 0) plus fractal value noise of +-5 m,
    quantised to 2^-10 m; 1-3 vents (seeded) near the summit; emission rates
    uniform in rate_range m^3/s for each of ``phases`` phases.
    Returns (z, vents [(x, y)], rates [nvents][phases])."""
    rng = SplitMix64(seed)
    ci, cj = (rows - 1) / 2.0, (cols - 1) / 2.0
    ii = np.arange(rows, dtype=np.float64)[:, None]
    jj = np.arange(cols, dtype=np.float64)[None, :]
    d = np.sqrt((ii - ci) ** 2 + (jj - cj) ** 2) * cell
    height = slope * min(rows, cols) / 2.0 * cell
    z = np.maximum(height - slope * d, 0.0) + 5.0 * _value_noise(rows, cols, seed * 7 + 1)
    z = quantise(np.maximum(z, 0.0))
    if nvents is None:
        nvents = 1 + int(rng.next_u64() % 3)
    spread = max(1.0, min(rows, cols) / 16.0)
    vents = []
    while len(vents) < nvents:
        vi = int(round(ci + rng.uniform(-spread, spread)))
        vj = int(round(cj + rng.uniform(-spread, spread)))
        if (vj, vi) not in vents:
            vents.append((vj, vi))
    rates = [[rng.uniform(*rate_range) for _ in range(phases)] for _ in range(nvents)]
    return np.ascontiguousarray(z), vents, rates


def sciara_scenarios(count: int, rows: int, cols: int, seed: int = 5, dems: int = 8, phases: int = 6,
                     emission_time: int = 3600):
    """``count`` SCIARA-fv2 scenarios for hazard mapping: ``dems`` synthetic
    volcanoes (sciara_inputs with seeds seed .. seed + dems - 1), scenario k
    on volcano k % dems with its own 1-3 vents near the summit and emission
    rates (SplitMix64 seeded by seed * 1009 + k).  Scenarios on the same
    volcano share its elevation array (read-only).  Returns [(z, vents,
    rates, emission_time)]."""
    zs = [sciara_inputs(rows, cols, seed=seed + d, phases=phases)[0] for d in range(min(dems, count))]
    ci, cj = (rows - 1) / 2.0, (cols - 1) / 2.0
    spread = max(1.0, min(rows, cols) / 16.0)
    out = []
    for k in range(count):
        rng = SplitMix64(seed * 1009 + k)
        nv = 1 + int(rng.next_u64() % 3)
        vents = []
        while len(vents) < nv:
            v = (int(round(cj + rng.uniform(-spread, spread))), int(round(ci + rng.uniform(-spread, spread))))
            if v not in vents:
                vents.append(v)
        rates = [[rng.uniform(10.0, 50.0) for _ in range(phases)] for _ in range(nv)]
        out.append((zs[k % len(zs)], vents, rates, emission_time))
    return out
