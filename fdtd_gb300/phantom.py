"""Synthetic inputs in the reference's file formats.

Writes ``input_params`` (fixed line order, fdtd.cu:547-620), ``mat_specs``
records (``code name sigma eps_s eps_i tau``, fdtd.cu:895) and PGM slices
``v1_%05d.pgm`` (``P2``, a two-token comment line, ``W H``, maxval, then the
codes x fastest; fdtd.cu:911-933), so the reference program and this library
read the same geometry.  Phantoms are seeded and deterministic.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np


@dataclass(frozen=True)
class Material:
    code: int
    name: str
    sigma: float
    eps_s: float
    eps_i: float
    tau: float


VACUUM = Material(0, "air", 0.0, 1.0, 1.0, 0.0)


@dataclass
class Config:
    """One solve in the reference's parameter terms (dx = c / f / epw)."""

    nx: int
    ny: int
    nz: int
    t_max: int
    env_dir: str = "pgm"
    output_dir: str = "output"
    elements_per_wavelength: int = 300
    wave_frequency: float = 1.0e9
    pulse_width: float = 0.5
    pulse_modulation_frequency: float = 1.0
    sources: list = field(default_factory=list)   # 0-based (x, y, z)
    default: Material = VACUUM


def write_input_params(path: str | os.PathLike, cfg: Config) -> None:
    """input_params in the reference's line order (1-based source indices)."""
    d = cfg.default
    lines = [
        f"nx_ny_nz: {cfg.nx} {cfg.ny} {cfg.nz}",
        f"t_max: {cfg.t_max}",
        "nf: 1",
        f"env_set_dir: {cfg.env_dir}",
        'env_file_prefix: "ver"',
        f"output_dir: {cfg.output_dir}",
        'output_format: "txt"',
        "impulse_resp_flag: 0",
        "pec_flag: 0",
        "read_env_flag: 0",
        "output_flag: 1",
        "bzip2_flag: 0",
        "output_start: 0 0 0",
        "output_finish: 0 0 0",
        "source_type: soft",
        f"elements_per_wavelength: {cfg.elements_per_wavelength}",
        f"wave_frequency: {cfg.wave_frequency:.9e}",
        f"pulse_width: {cfg.pulse_width:.9g}",
        f"pulse_modulation_frequency: {cfg.pulse_modulation_frequency:.9g}",
        f"number_of_excitation_sources: {len(cfg.sources)}",
    ]
    lines += [f"source_location: {x + 1} {y + 1} {z + 1}" for (x, y, z) in cfg.sources]
    lines += [
        "pulse_type: 2",
        f"fsigma: {d.sigma:.9g}",
        f"feps_s: {d.eps_s:.9g}",
        f"feps_inf: {d.eps_i:.9g}",
        f"ftau_d: {d.tau:.9e}",
    ]
    Path(path).write_text("\n".join(lines) + "\n")


def write_mat_specs(path: str | os.PathLike, materials: list[Material]) -> None:
    rows = [f"{m.code} {m.name}\t{m.sigma:.8f}\t{m.eps_s:.8f}\t{m.eps_i:.8f}\t{m.tau:.8E}" for m in materials]
    rows += ["", "! <mcode> <mdesc> <sigma> <eps_s> <eps_i> <tau_1>"]
    Path(path).write_text("\n".join(rows) + "\n")


def write_pgm_slices(directory: str | os.PathLike, codes: np.ndarray) -> None:
    """codes: (nz, ny, nx) uint8; one file per z plane, 1-based names."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    nz, ny, nx = codes.shape
    maxval = int(codes.max()) if codes.size else 0
    digits = np.array([str(i) for i in range(256)], dtype=object)
    for z in range(nz):
        plane = digits[codes[z]]
        body = "\n".join(" ".join(row) for row in plane)
        (d / f"v1_{z + 1:05d}.pgm").write_text(f"P2\n# test\n{nx} {ny}\n{maxval}\n{body}\n")


def specs_table(materials: list[Material], n: int = 256) -> np.ndarray:
    t = np.zeros((n, 4), np.float32)
    for m in materials:
        t[m.code] = (m.sigma, m.eps_s, m.eps_i, m.tau)
    return t


# --------------------------------------------------------------- phantoms

def sphere_phantom(n: int = 64, radius: float = 16.0, code: int = 1) -> np.ndarray:
    """Vacuum cube with one centred sphere (the 64^3 plain FP32 case)."""
    z, y, x = np.mgrid[0:n, 0:n, 0:n]
    c = (n - 1) / 2.0
    inside = (x - c) ** 2 + (y - c) ** 2 + (z - c) ** 2 <= radius ** 2
    out = np.zeros((n, n, n), np.uint8)
    out[inside] = code
    return out


SPHERE_MATERIAL = Material(1, "debye_sphere", 0.5, 50.0, 4.0, 8.0e-12)


def ellipsoid_phantom(shape: tuple[int, int, int], n_shells: int = 8, seed: int = 0,
                      semi_min: float = 60.0, semi_max: float = 230.0, jitter: float = 0.10):
    """Nested, randomly scaled ellipsoids (outermost first) around the centre;
    shell k gets class k+1.  Returns (codes, materials, outer semi-axes)."""
    nz, ny, nx = shape
    rng = np.random.default_rng(seed)
    base = np.linspace(semi_max, semi_min, n_shells)
    # keep a margin of vacuum to the Mur faces: 24 cells, or 1/8 of a small axis
    half = np.array([nx, ny, nz], np.float64) / 2
    room = np.maximum(half - np.minimum(24.0, np.floor(2 * half / 8)), 1.0)
    axes = []
    for b in base:
        a = b * (1.0 + rng.uniform(-jitter, jitter, 3))
        axes.append(np.maximum(np.minimum(a, room), 1.0))
    cx, cy, cz = (nx - 1) / 2, (ny - 1) / 2, (nz - 1) / 2
    codes = np.zeros(shape, np.uint8)
    xs = ((np.arange(nx) - cx) ** 2)[None, None, :]
    ys = ((np.arange(ny) - cy) ** 2)[None, :, None]
    for z in range(nz):
        zz = (z - cz) ** 2
        plane = codes[z]
        for k, (ax, ay, az) in enumerate(axes):
            inside = xs[0] / ax ** 2 + ys[0] / ay ** 2 + zz / az ** 2 <= 1.0
            plane[inside] = k + 1
    mats = [VACUUM]
    for k in range(n_shells):
        eps_i = rng.uniform(4, 40)
        eps_s = rng.uniform(max(eps_i, 10), 80)
        tau = rng.uniform(5e-12, 15e-12)
        sigma = rng.uniform(0.05, 2.0)
        mats.append(Material(k + 1, f"tissue_{k + 1}", sigma, eps_s, eps_i, tau))
    return codes, mats, axes[0]


def c1_inputs(root: str | os.PathLike, n: int = 64, t_max: int = 500) -> Path:
    """Writes the 64^3 sphere case under root; returns the input_params path."""
    root = Path(root)
    root.mkdir(parents=True, exist_ok=True)
    codes = sphere_phantom(n, radius=16.0 * n / 64.0)
    write_pgm_slices(root / "pgm", codes)
    write_mat_specs(root / "mat_specs", [VACUUM, SPHERE_MATERIAL])
    cfg = Config(n, n, n, t_max, env_dir=str(root / "pgm"), output_dir=str(root / "out"),
                 sources=[(n // 4, n // 2, n // 2)])
    write_input_params(root / "input_params", cfg)
    return root / "input_params"


def c2_config(shape=(400, 512, 512), seed: int = 0):
    """512 x 512 x 400 nested-ellipsoid phantom, 900 MHz z-dipole 20 cells
    outside the outer shell.  Returns (codes, materials, Config)."""
    nz, ny, nx = shape
    codes, mats, outer = ellipsoid_phantom(shape, seed=seed)
    cx, cy, cz = (nx - 1) // 2, (ny - 1) // 2, (nz - 1) // 2
    sx = int(round(cx - outer[0] - 20))
    sources = [(max(sx, 1), cy, cz + dz) for dz in (-1, 0, 1)]
    cfg = Config(nx, ny, nz, 3000, wave_frequency=1.0e9, elements_per_wavelength=300,
                 pulse_width=0.5, pulse_modulation_frequency=0.9, sources=sources)
    return codes, mats, cfg
