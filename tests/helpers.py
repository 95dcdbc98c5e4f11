"""Shared helpers for the tests: golden-run loading and field comparison."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from oracle import pyoracle as po

GOLDEN = Path(__file__).resolve().parent / "golden"
RUNS = ["random17x9x11", "sphere24", "classes70x20x9"]

# Parity bound of the FP32 CUDA path against the reference FP32 kernels (and
# the FP32 oracle that reproduces them bit for bit): relative L2 per field.
REL_L2_TOL = 1e-5


@dataclass
class GoldenRun:
    name: str
    dims: tuple[int, int, int]
    steps: int
    consts: dict
    sources: list
    jz: np.ndarray
    media: po.Media
    state: list            # 21 arrays after `steps` steps (reference slots)
    codes: np.ndarray | None
    specs: np.ndarray | None

    def cfg(self, corrected: bool = False, jz: np.ndarray | None = None):
        return po.make_cfg(self.dims, self.jz if jz is None else jz, sources=self.sources, corrected=corrected,
                           consts=self.consts)

    def latest(self) -> dict[str, np.ndarray]:
        """E, D of the last step and H, from the reference slot layout."""
        k = (self.steps - 1) % 3
        out = {"hx": self.state[0], "hy": self.state[1], "hz": self.state[2]}
        for c, n in enumerate("xyz"):
            out["e" + n] = self.state[3 + 3 * k + c]
            out["d" + n] = self.state[12 + 3 * k + c]
        return out


def load_run(name: str) -> GoldenRun:
    z = np.load(GOLDEN / f"run_{name}.npz")
    nx, ny, nz = (int(v) for v in z["dims"])
    c = z["consts"]
    consts = dict(dt=float(c[0]), dx=float(c[1]), dy=float(c[2]), dz=float(c[3]), mu0=float(c[4]), eps0=float(c[5]))
    media = po.Media(z["sigma"], z["eps_i"], z["eps_s"], z["tau_d"])
    rp, off = [], 0
    for s in po.rp_shapes(nx, ny, nz):
        n = int(np.prod(s))
        rp.append(z["rp"][off:off + n].reshape(s).copy())
        off += n
    media.rp = rp
    return GoldenRun(name=name, dims=(nx, ny, nz), steps=int(z["steps"]), consts=consts,
                     sources=[tuple(int(v) for v in s) for s in z["sources"]], jz=z["jz"].astype(np.float32),
                     media=media, state=[z[f"s{i}"] for i in range(21)],
                     codes=z["codes"] if "codes" in z else None, specs=z["specs"] if "specs" in z else None)


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    if den == 0.0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / den)


def assert_fields_close(got: dict, want: dict, tol: float = REL_L2_TOL, names=None) -> None:
    names = names or sorted(want)
    errs = {n: rel_l2(got[n], want[n]) for n in names}
    bad = {n: e for n, e in errs.items() if not e <= tol}
    assert not bad, f"relative L2 above {tol}: {bad} (all: {errs})"


def bits_equal(a: np.ndarray, b: np.ndarray) -> bool:
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def class_media(codes: np.ndarray, specs: np.ndarray, rp) -> po.Media:
    m = po.Media(sigma=np.ascontiguousarray(specs[codes, 0]), eps_i=np.ascontiguousarray(specs[codes, 2]),
                 eps_s=np.ascontiguousarray(specs[codes, 1]), tau_d=np.ascontiguousarray(specs[codes, 3]))
    m.rp = rp
    return m


def random_case(nx: int, ny: int, nz: int, seed: int, ncls: int = 5, nsrc: int = 2):
    """Class-coded random Debye media, random Mur slabs and sources."""
    rng = np.random.default_rng(seed)
    specs = np.zeros((ncls, 4), np.float32)
    specs[0] = (0.0, 1.0, 1.0, 0.0)
    for k in range(1, ncls):
        specs[k] = (rng.uniform(0.05, 2), rng.uniform(10, 80), rng.uniform(4, 10), rng.uniform(5e-12, 15e-12))
    codes = rng.integers(0, ncls, size=(nz, ny, nx)).astype(np.uint8)
    rp = [rng.uniform(1, 3, s).astype(np.float32) for s in po.rp_shapes(nx, ny, nz)]
    sources = [(int(rng.integers(1, nx)), int(rng.integers(1, ny)), int(rng.integers(0, nz))) for _ in range(nsrc)]
    consts = dict(dt=1.9245009e-12, dx=1e-3, dy=1e-3, dz=1e-3, mu0=1.2566371e-06, eps0=8.841941e-12)
    jz = (rng.standard_normal(256) * 0.5).astype(np.float32)
    return codes, specs, rp, sources, consts, jz
