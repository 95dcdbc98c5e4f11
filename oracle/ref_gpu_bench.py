"""Times the reference's own CUDA kernels on this GPU (measurement
infrastructure, not the product).

The reference kernel file compiled for sm_103a (``oracle/_ref/ref_kernels.cubin``)
runs the 512 x 512 x 400 Debye phantom through its five kernels per step with
the reference's launch grid and slot rotation, snapshot output gated off, on
one stream; CUDA events bracket the timed steps.  The library's single-pass
and compact solvers run the same workload in the same process for a
same-GPU comparison.  Step indices stay below 512, the window in which the
reference's 512-entry dJz table is defined.

    python -m oracle.ref_gpu_bench [--dims NX NY NZ] [--steps K] [--warmup W]
"""
from __future__ import annotations

import argparse
import json
import tempfile
from pathlib import Path

import numpy as np

from . import pyoracle as po


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", type=int, nargs=3, default=[512, 512, 400])
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=6)
    args = ap.parse_args()
    if args.warmup + args.steps > 510:
        raise SystemExit("warmup + steps must stay below 511 (the reference's dJz window)")
    import fdtd_gb300 as fg
    from fdtd_gb300 import phantom as ph

    nx, ny, nz = args.dims
    cells = nx * ny * nz
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        codes, mats, cfg = ph.c2_config((nz, ny, nx))
        cfg.env_dir = str(tmp / "pgm")
        cfg.output_dir = str(tmp / "out")
        ph.write_input_params(tmp / "input_params", cfg)
        ph.write_mat_specs(tmp / "mat_specs", mats)
        p = fg.Params.read(tmp / "input_params")
        specs = fg.read_specs(tmp / "mat_specs")[: len(mats)]
        q = po.params_read(tmp / "input_params", "f32")

    jz = p.setup_sources()
    media = po.Media(*(np.ascontiguousarray(specs[codes, k]) for k in (0, 2, 1, 3)))
    media.rp = po.uniform_media(q).rp
    ms = po.ref_gpu_run(po.make_cfg(q, jz), media, args.steps, warmup=args.warmup)
    out = {"what": "reference CUDA kernels (fdtd_calculations.cu, nvcc defaults, sm_103a) vs this library, "
                   "same GPU, same process",
           "workload": f"nested-ellipsoid Debye phantom {nx}x{ny}x{nz}", "steps": args.steps,
           "warmup": args.warmup, "reference_gpu": {"ms_per_step": ms / args.steps,
                                                    "cell_updates_per_s": cells * args.steps / (ms / 1e3)}}
    del media
    import torch

    for name, kernel in (("single_pass", fg.KERNEL_SINGLE_PASS), ("compact", fg.KERNEL_COMPACT)):
        with fg.Solver(p, codes, specs, kernel=kernel) as s:
            s.run(args.warmup)
            s.synchronize()
            stream = torch.cuda.ExternalStream(s.stream)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            s.run(args.steps)
            b.record(stream)
            s.synchronize()
            t = a.elapsed_time(b)
        out[name] = {"ms_per_step": t / args.steps, "cell_updates_per_s": cells * args.steps / (t / 1e3),
                     "speedup_vs_reference_gpu": ms / t}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
