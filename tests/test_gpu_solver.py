"""Solver handle (graph-replayed step loop, snapshots) against the golden runs
and the FP64 oracle, driven from the reference's input files."""
from __future__ import annotations

import numpy as np
import pytest

import fdtd_gb300 as fg
from fdtd_gb300 import phantom as ph
from oracle import pyoracle as po

from .helpers import REL_L2_TOL, assert_fields_close, load_run, rel_l2

pytestmark = pytest.mark.gpu

KERNELS = [fg.KERNEL_SINGLE_PASS, fg.KERNEL_TWO_PASS]


def solver_from_files(root, n, t_max, kernel, scheme=fg.SCHEME_REFERENCE, timeskip=None):
    path = ph.c1_inputs(root, n=n, t_max=t_max)
    p = fg.Params.read(path)
    if timeskip is not None:
        p.set_timeskip(timeskip)
    codes = fg.load_material_codes(p, root / "pgm")
    specs = fg.read_specs(root / "mat_specs")
    return p, codes, specs, fg.Solver(p, codes, specs, scheme=scheme, kernel=kernel, nclasses=2)


@pytest.mark.parametrize("kernel", KERNELS)
def test_solver_from_reference_files_matches_reference_run(cuda, tmp_path, kernel):
    g = load_run("sphere24")
    p, codes, specs, s = solver_from_files(tmp_path, 24, 60, kernel)
    assert np.array_equal(codes, g.codes)
    for chunk in (5, 17, 26):  # uneven chunks exercise both graph parities
        s.run(chunk)
    assert s.steps == g.steps == 48
    assert_fields_close(s.fields(), g.latest())
    s.close()


@pytest.mark.parametrize("kernel", KERNELS)
def test_snapshots_equal_field_reads(cuda, tmp_path, kernel):
    p, codes, specs, a = solver_from_files(tmp_path / "a", 20, 30, kernel)
    got = {}
    a.set_snapshots(every=5, fields=("ex", "hz", "dz"), z0=3, nplanes=4,
                    callback=lambda step, name, data: got.__setitem__((step, name), data))
    a.run(23)
    a.flush_snapshots()
    assert sorted({k[0] for k in got}) == [0, 5, 10, 15, 20]
    _, _, _, b = solver_from_files(tmp_path / "b", 20, 30, kernel)
    done = 0
    for step in (0, 5, 10, 15, 20):
        b.run(step + 1 - done)
        done = step + 1
        for name in ("ex", "hz", "dz"):
            assert np.array_equal(got[(step, name)], b.field(name)[3:7]), (step, name)
    a.close()
    b.close()


def test_text_snapshots_in_reference_layout(cuda, tmp_path):
    p, codes, specs, s = solver_from_files(tmp_path, 12, 9, fg.KERNEL_SINGLE_PASS)
    out = tmp_path / "out"
    out.mkdir()
    s.set_snapshots(every=1, fields=fg.FIELDS, output_dir=out)
    s.run(3)
    s.flush_snapshots()
    names = sorted(q.name for q in out.iterdir())
    assert len(names) == 3 * 9 * 12
    assert names[0] == "D_field_x_00000_z00000.out"
    ez = s.field("ez")
    text = (out / "E_field_z_00002_z00006.out").read_text()
    want = "".join("".join(" % 9.3E" % float(v) for v in row) + "\n" for row in ez[6])
    assert text == want
    s.close()


def test_c1_sphere_corrected_scheme_500_steps_vs_fp64_oracle(cuda, tmp_path):
    """64^3 sphere, dt = 0.99 of the Courant limit, corrected Debye scheme,
    501 steps: relative L2 of every field against the FP64 oracle."""
    p, codes, specs, s = solver_from_files(tmp_path, 64, 500, fg.KERNEL_SINGLE_PASS, scheme=fg.SCHEME_CORRECTED,
                                           timeskip=0.99)
    steps = p.iterationsCount
    assert steps == 501
    s.run(steps)
    got = s.fields()
    s.close()
    q = po.params_read(tmp_path / "input_params", "f64")
    q.dt = p.dt
    jz = p.setup_sources()
    media = po.Media(*(np.ascontiguousarray(specs[codes, k]) for k in (0, 2, 1, 3)))
    media.rp = po.uniform_media(q).rp
    cfg = po.make_cfg(q, jz, corrected=True)
    st = po.State(64, 64, 64, np.float64)
    po.run(cfg, media, st, 0, steps)
    want = st.latest(steps)
    assert all(np.all(np.isfinite(v)) for v in want.values())
    assert max(np.abs(v).max() for v in want.values()) > 0
    assert_fields_close(got, want, tol=REL_L2_TOL)


def test_c1_sphere_reference_scheme_finite_window(cuda, tmp_path):
    """Reference scheme on the 64^3 sphere: identical to the FP32 oracle
    (which reproduces the reference kernels) while the fields are finite."""
    p, codes, specs, s = solver_from_files(tmp_path, 64, 60, fg.KERNEL_SINGLE_PASS)
    s.run(60)
    got = s.fields()
    s.close()
    q = po.params_read(tmp_path / "input_params", "f32")
    jz = p.setup_sources()
    media = po.Media(*(np.ascontiguousarray(specs[codes, k]) for k in (0, 2, 1, 3)))
    media.rp = po.uniform_media(q).rp
    st = po.State(64, 64, 64, np.float32)
    po.run(po.make_cfg(q, jz), media, st, 0, 60)
    want = st.latest(60)
    assert all(np.all(np.isfinite(v)) for v in want.values())
    assert_fields_close(got, want)


def test_drop_in_executable_writes_reference_layout(cuda, tmp_path):
    """fdtd_gb300/bin/fdtd reads input_params / mat_specs / PGM slices like the
    reference program and writes every field every step (writeResults3d
    layout); its Ez after the last step equals the solver's."""
    import subprocess

    n = 12
    path = ph.c1_inputs(tmp_path, n=n, t_max=3)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(fg.EXE_PATH), "--params", str(path), "--specs", str(tmp_path / "mat_specs")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    names = sorted(q.name for q in out.iterdir())
    assert len(names) == 3 * 9 * n  # 3 steps, 9 fields, n planes
    p, codes, specs, s = solver_from_files(tmp_path / "again", n, 3, fg.KERNEL_SINGLE_PASS)
    s.run(3)
    ez = s.field("ez")
    s.close()
    for z in (0, 5, n - 1):
        text = (out / f"E_field_z_00002_z{z:05d}.out").read_text()
        want = "".join("".join(" % 9.3E" % float(v) for v in row) + "\n" for row in ez[z])
        assert text == want


def test_binary_snapshots_hold_the_exact_fields(cuda, tmp_path):
    """Text and binary side by side: each .f32 file holds the planes' floats
    bit for bit, and the text files of the same step format those values."""
    p, codes, specs, s = solver_from_files(tmp_path, 20, 9, fg.KERNEL_SINGLE_PASS)
    out = tmp_path / "snap"
    out.mkdir()
    s.set_snapshots(every=3, fields=("ez", "hx", "dy"), z0=5, nplanes=4, output_dir=out,
                    format=fg.SNAPSHOT_TEXT_AND_BINARY)
    s.run(7)  # snapshots after steps 0, 3, 6
    s.flush_snapshots()
    want = s.fields()
    s.close()
    for name, tag in (("ez", "E_field_z"), ("hx", "H_field_x"), ("dy", "D_field_y")):
        raw = np.fromfile(out / f"{tag}_00006_z00005_n00004.f32", dtype="<f4").reshape(4, 20, 20)
        assert np.array_equal(raw.view(np.uint32), want[name][5:9].view(np.uint32)), name
        text = (out / f"{tag}_00006_z00007.out").read_text()
        assert text == "".join("".join(" % 9.3E" % float(v) for v in row) + "\n" for row in raw[2])
    assert len(list(out.glob("*.f32"))) == 3 * 3
    assert len(list(out.glob("*.out"))) == 3 * 3 * 4


def test_drop_in_voxel_cache_and_compact_binary_output(cuda, tmp_path):
    """The drop-in with --voxel-cache: the first run parses the slices and
    writes the cache, the second reads it; with --kernel compact --format
    binary --fields ez both runs write the same Ez bits, equal to the
    compact solver's."""
    import subprocess

    n = 16
    path = ph.c1_inputs(tmp_path, n=n, t_max=6)
    cache = tmp_path / "voxels.u8v"
    runs = []
    for k in range(2):
        out = tmp_path / "out"
        if out.exists():
            for q in out.iterdir():
                q.unlink()
        else:
            out.mkdir()
        r = subprocess.run([str(fg.EXE_PATH), "--params", str(path), "--specs", str(tmp_path / "mat_specs"),
                            "--kernel", "compact", "--format", "binary", "--fields", "ez",
                            "--voxel-cache", str(cache)], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert ("voxels from cache" if k else "voxel cache written") in r.stdout, r.stdout
        files = sorted(out.glob("*.f32"))
        assert len(files) == 6 and not list(out.glob("*.out"))
        runs.append(np.fromfile(out / f"E_field_z_00005_z00000_n{n:05d}.f32", dtype="<f4").reshape(n, n, n))
    assert np.array_equal(runs[0].view(np.uint32), runs[1].view(np.uint32))
    p, codes, specs, s = solver_from_files(tmp_path / "again", n, 6, fg.KERNEL_COMPACT)
    s.run(6)
    ez = s.field("ez")
    s.close()
    assert np.array_equal(runs[1].view(np.uint32), ez.view(np.uint32))


def test_drop_in_compact16_binary_output_equals_the_solver(cuda, tmp_path):
    """The drop-in with --kernel compact16 writes H and E only (no D files)
    and its Ez bits equal the 16-bit-R solver's."""
    import subprocess

    n = 16
    path = ph.c1_inputs(tmp_path, n=n, t_max=6)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(fg.EXE_PATH), "--params", str(path), "--specs", str(tmp_path / "mat_specs"),
                        "--kernel", "compact16", "--format", "binary"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert not list(out.glob("D_field_*")) and len(list(out.glob("E_field_z_*.f32"))) == 6
    got = np.fromfile(out / f"E_field_z_00005_z00000_n{n:05d}.f32", dtype="<f4").reshape(n, n, n)
    p, codes, specs, s = solver_from_files(tmp_path / "again", n, 6, fg.KERNEL_COMPACT_R16)
    s.run(6)
    ez = s.field("ez")
    s.close()
    assert np.array_equal(got.view(np.uint32), ez.view(np.uint32))


@pytest.mark.parametrize("kernel", [fg.KERNEL_SINGLE_PASS, fg.KERNEL_COMPACT_R16])
def test_class_rows_beyond_the_material_change_nothing(cuda, tmp_path, kernel):
    """The solve keeps the specs rows up to the largest class present: every
    row of the table given, or just the two the sphere uses, same bits; a
    class index at or above the rows given is refused."""
    path = ph.c1_inputs(tmp_path, n=20, t_max=30)
    p = fg.Params.read(path)
    codes = fg.load_material_codes(p, tmp_path / "pgm")
    specs = fg.read_specs(tmp_path / "mat_specs")
    assert len(specs) == fg.MAX_CLASSES and codes.max() == 1
    out = {}
    for rows in (2, None):
        with fg.Solver(p, codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=kernel, nclasses=rows) as s:
            s.run(25)
            out[rows] = s.fields()
    for name in out[2]:
        assert np.array_equal(out[2][name], out[None][name]), name
    with pytest.raises(fg.FdtdError):
        fg.Solver(p, codes, specs, scheme=fg.SCHEME_CORRECTED, kernel=kernel, nclasses=1)


def test_field_into_a_caller_buffer(cuda, tmp_path):
    p, codes, specs, s = solver_from_files(tmp_path, 20, 30, fg.KERNEL_SINGLE_PASS)
    s.run(12)
    buf = np.full(p.shape, np.nan, np.float32)
    assert s.field("ez", out=buf) is buf
    assert np.array_equal(buf, s.field("ez"))
    with pytest.raises(ValueError):
        s.field("ez", out=np.empty(p.shape, np.float64))
    s.close()
