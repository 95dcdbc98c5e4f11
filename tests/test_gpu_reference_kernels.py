"""The reference's own CUDA kernels, compiled for sm_103a and run on the GPU
through the oracle harness, against the CPU oracle and against this
library's kernels on the same inputs (step indices below 512, the window in
which the reference's 512-entry dJz is defined)."""
from __future__ import annotations

import numpy as np
import pytest

import fdtd_gb300 as fg
from fdtd_gb300 import phantom as ph
from oracle import pyoracle as po

from .gpu_util import Params, make_params
from .helpers import assert_fields_close, class_media, random_case

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not po.ref_gpu_available(), reason="reference kernels were not compiled")]


def _sphere_inputs(root, n, t_max):
    path = ph.c1_inputs(root, n=n, t_max=t_max)
    p = fg.Params.read(path)
    codes = fg.load_material_codes(p, root / "pgm")
    specs = fg.read_specs(root / "mat_specs")
    q = po.params_read(root / "input_params", "f32")
    jz = p.setup_sources()
    media = po.Media(*(np.ascontiguousarray(specs[codes, k]) for k in (0, 2, 1, 3)))
    media.rp = po.uniform_media(q).rp
    return p, codes, specs, po.make_cfg(q, jz), media


def test_reference_gpu_kernels_match_cpu_oracle_and_solver(cuda, tmp_path):
    """64^3 sphere, 60 steps: reference kernels on the GPU vs the FP32 oracle
    (which reproduces them on the CPU bit for bit) and vs the single-pass
    solver.  GPU and CPU differ only in the compiler's contraction of a*b+c
    into fused multiply-adds."""
    p, codes, specs, cfg, media = _sphere_inputs(tmp_path, 64, 60)
    st = po.State(64, 64, 64, np.float32)
    po.ref_gpu_run(cfg, media, 60, state=st)
    ref_gpu = st.latest(60)
    assert max(np.abs(v).max() for v in ref_gpu.values()) > 0
    cpu = po.State(64, 64, 64, np.float32)
    po.run(cfg, media, cpu, 0, 60)
    assert_fields_close(ref_gpu, cpu.latest(60))
    with fg.Solver(p, codes, specs, nclasses=2) as s:
        s.run(60)
        assert_fields_close(s.fields(), ref_gpu)


@pytest.mark.parametrize("dims", [(37, 29, 23), (130, 20, 12)])
def test_reference_gpu_kernels_ragged_grid(cuda, dims):
    """nx not a multiple of the reference's 128-thread blocks, random Debye
    classes and Mur slabs, two sources; the compat launchers take the same
    float arrays."""
    steps = 45
    codes, specs, rp, sources, consts, jz = random_case(*dims, seed=11, ncls=4, nsrc=2)
    media = class_media(codes, specs, rp)
    cfg = po.make_cfg(dims, jz, sources=sources, consts=consts)
    st = po.State(*dims, np.float32)
    po.ref_gpu_run(cfg, media, steps, state=st)
    cpu = po.State(*dims, np.float32)
    po.run(cfg, media, cpu, 0, steps)
    assert_fields_close(st.latest(steps), cpu.latest(steps))


def test_reference_gpu_refuses_steps_past_the_jz_table(cuda, tmp_path):
    p, codes, specs, cfg, media = _sphere_inputs(tmp_path, 16, 9)
    with pytest.raises(RuntimeError):
        po.ref_gpu_run(cfg, media, 600)
