"""The drop-in process contract on the GPU: fluidsim CLI, VTK files, fields
set/get through host buffers."""
import os
import subprocess

import numpy as np
import pytest

from fluidsim_gb300 import api, build, cases

pytestmark = pytest.mark.gpu

INI = """[physics]
gravity = 9.81
[fluid]
is_viscid = true
fluid_density = 1000
fluid_sound_speed = 30
[solid]
solid_density = 1100
youngs_modulus = 1e6
poisson_ratio = 0.4
[domain]
xmin = 0
xmax = 0.24
ymin = 0
ymax = 0.16
zmin = 0
zmax = 0.16
[time]
dt = 1e-4
istart = 0
iend = 4
solid_sub_step = 4
result_interval = 2
[kernel]
smoothing_length = 0.013
particle_diameter = 0.01
impact_length_hsml_ratio = 2.0
"""


def _vtk_text(title, pos, name, values, vector):
    n = len(pos)
    s = "# vtk DataFile Version 2.0\n%s\nASCII\nDATASET POLYDATA\nPOINTS %d float\n" % (title, n)
    s += "".join("%f %f %f\n" % tuple(float(v) for v in p) for p in pos)
    s += "POINT_DATA %d\n" % n
    if vector:
        s += "VECTORS %s float\n" % name
        s += "".join("%f %f %f\n" % tuple(float(v) for v in p) for p in values)
    else:
        s += "SCALARS %s float 1\nLOOKUP_TABLE default\n" % name
        s += "".join("%f\n" % float(v) for v in values)
    return s


def test_vtk_files_match_reference_format(tmp_path):
    cfg, pa = cases.make(cases.tiny_box())
    with api.Simulation(cfg, pa, device=0) as sim:
        sim.step(2)
        sim.sync()
        sim.write_vtk(str(tmp_path), 7)
        fpos, fvel, frho = sim.get("fluid_pos"), sim.get("fluid_vel"), sim.get("fluid_rho")
        vpos, vp = sim.get("virt_pos"), sim.get("virt_p")
        spos = sim.get("solid_pos")
    d = tmp_path
    assert (d / "fluid" / "fluid_velocity-7.vtk").read_text() == _vtk_text("Velocity vector file", fpos,
                                                                            "velocity", fvel, True)
    assert (d / "fluid" / "fluid_density-7.vtk").read_text() == _vtk_text("scalar vector file", fpos, "density",
                                                                           frho, False)
    # the reference writes its always-zero color array as "pressure"
    assert (d / "fluid" / "fluid_pressure-7.vtk").read_text() == _vtk_text("scalar vector file", fpos, "pressure",
                                                                            np.zeros(len(fpos)), False)
    assert (d / "virtual" / "virt_pressure-7.vtk").read_text() == _vtk_text("scalar vector file", vpos, "pressure",
                                                                             vp, False)
    assert (d / "solid" / "solid_density-7.vtk").read_text() == _vtk_text("scalar vector file", spos, "density",
                                                                           np.full(len(spos), 1100.0), False)
    for f in ("fluid/fluid_true_pressure-7.vtk", "solid/solid_velocity-7.vtk", "solid/solid_pressure-7.vtk",
              "solid/solid_normal-7.vtk", "virtual/virt_normal-7.vtk"):
        assert (d / f).exists(), f


def test_cli_process_contract(tmp_path):
    build.build()
    cfg_dir, data, out = tmp_path / "config", tmp_path / "data", tmp_path / "out"
    cfg_dir.mkdir()
    (cfg_dir / "input.ini").write_text(INI)
    cfg = api.config_from_ini(str(cfg_dir / "input.ini"))
    _, pa = cases.make((cfg, cases.tiny_box()[1]))
    pa.write_dat(str(data))
    r = subprocess.run([build.CLI, "--config", str(cfg_dir / "input.ini"), "--data", str(data), "--out", str(out)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    # iend = 4, result_interval = 2: output before steps 1 and 3, and after the loop
    for k in (0, 1, 2):
        assert (out / "fluid" / ("fluid_density-%d.vtk" % k)).exists(), k
    assert not (out / "fluid" / "fluid_density-3.vtk").exists()
    # the final file equals 4 steps through the library
    with api.Simulation(cfg, api.read_dat(str(data)), device=0) as sim:
        sim.step(4)
        sim.sync()
        want = _vtk_text("scalar vector file", sim.get("fluid_pos"), "density", sim.get("fluid_rho"), False)
    assert (out / "fluid" / "fluid_density-2.vtk").read_text() == want


def test_cli_reports_bad_input(tmp_path):
    build.build()
    (tmp_path / "input.ini").write_text("xmax = 1\n")
    r = subprocess.run([build.CLI, "--config", str(tmp_path / "input.ini"), "--data", str(tmp_path)],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "FSIM_EINVAL" in r.stderr


def test_set_get_round_trip_and_pinned():
    cfg, pa = cases.make(cases.tiny_box(jitter=0.01, seed=1))
    with api.Simulation(cfg, pa, device=0) as sim:
        sim.step(3)
        sim.sync()
        for k in ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel"):
            a = sim.get(k)
            b = api.PinnedBuffer(a.shape)
            b.array[...] = a * 0.5 + 0.25
            sim.set_ptr(k, b.ptr, b.nbytes)
            c = sim.get(k)
            assert np.array_equal(c, b.array), k
            b.free()
        with pytest.raises(api.FsimError):
            sim.set("virt_p", np.zeros(pa.n_virt, np.float32))
        with pytest.raises(api.FsimError):
            sim.set("fluid_rho", np.zeros(3, np.float32))


def test_unsorted_fields_rejected_until_phase_runs():
    cfg, pa = cases.make(cases.tiny_box())
    with api.Simulation(cfg, pa, device=0) as sim:
        sim.phase(api.PHASE_CELL)
        with pytest.raises(api.FsimError):
            sim.get("solid_normal")  # stale until the coupling phase runs
        sim.phase(api.PHASE_COUPLE)
        assert np.isfinite(sim.get("solid_normal")).all()
        with pytest.raises(api.FsimError):
            sim.get("fluid_drho_dt")  # keep_derivatives is off


def _read_binary_vtk(path):
    """Parse a BINARY legacy-VTK polydata file with one point-data array."""
    data = path.read_bytes()
    head_end = data.index(b"float\n", data.index(b"POINTS")) + len(b"float\n")
    header = data[:head_end].decode()
    assert header.split("\n")[2] == "BINARY"
    n = int(header.split("POINTS ")[1].split()[0])
    pts = np.frombuffer(data, ">f4", 3 * n, head_end).reshape(n, 3)
    rest = data[head_end + 12 * n + 1:]
    line_end = rest.index(b"\n", rest.index(b"\n") + 1) + 1  # POINT_DATA + VECTORS/SCALARS lines
    kind = rest[:line_end].decode()
    if "LOOKUP_TABLE" in rest[line_end:line_end + 30].decode(errors="ignore"):
        line_end = rest.index(b"\n", line_end) + 1
        return pts, np.frombuffer(rest, ">f4", n, line_end), kind
    return pts, np.frombuffer(rest, ">f4", 3 * n, line_end).reshape(n, 3), kind


def test_binary_vtk_holds_exact_fields(tmp_path):
    cfg, pa = cases.make(cases.tiny_box(jitter=0.01, seed=8))
    with api.Simulation(cfg, pa, device=0) as sim:
        sim.step(2)
        sim.sync()
        sim.write_vtk(str(tmp_path), 3, binary=True)
        pos, vel, rho, p = (sim.get(f) for f in ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p"))
        spos = sim.get("solid_pos")
    d = tmp_path / "fluid"
    x, v, kind = _read_binary_vtk(d / "fluid_velocity-3.vtk")
    assert "VECTORS velocity float" in kind
    assert np.array_equal(x, pos) and np.array_equal(v, vel)
    x, r, kind = _read_binary_vtk(d / "fluid_density-3.vtk")
    assert "SCALARS density float 1" in kind and np.array_equal(r, rho)
    _, tp, _ = _read_binary_vtk(d / "fluid_true_pressure-3.vtk")
    assert np.array_equal(tp, p)
    _, zero, _ = _read_binary_vtk(d / "fluid_pressure-3.vtk")
    assert not zero.any()
    xs, _, _ = _read_binary_vtk(tmp_path / "solid" / "solid_velocity-3.vtk")
    assert np.array_equal(xs, spos)


def test_many_fields_equal_single_fields():
    """fsim_get_fields / fsim_set_fields move the same bytes as the one-field calls."""
    cfg, pa = cases.make(cases.tiny_box(jitter=0.01, seed=6))
    names = ("fluid_pos", "fluid_vel", "fluid_rho", "fluid_p", "solid_pos", "solid_vel")
    with api.Simulation(cfg, pa, device=0) as sim:
        sim.step(2)
        sim.sync()
        single = {k: sim.get(k) for k in names}
        bufs = {k: api.PinnedBuffer(single[k].shape) for k in names}
        sim.get_many_ptr(names, [bufs[k].ptr for k in names], [bufs[k].nbytes for k in names])
        for k in names:
            assert np.array_equal(bufs[k].array, single[k]), k
        # set: perturb and write back all at once; read back one by one
        for k in names:
            bufs[k].array[...] = single[k] * 1.001
        sim.set_many_ptr(names, [bufs[k].ptr for k in names], [bufs[k].nbytes for k in names])
        for k in names:
            assert np.array_equal(sim.get(k), bufs[k].array), k
        for b in bufs.values():
            b.free()


def test_time_phases_reports_every_phase():
    cfg, pa = cases.make(cases.small_dam_break())
    with api.Simulation(cfg, pa, device=0) as sim:
        sim.step(2)
        ph = sim.time_phases(3)
        assert set(ph) == {"cell", "couple", "virt", "fluid", "solid"}
        assert all(v > 0 for v in ph.values())
        sim.step(1)  # timing steps are ordinary steps
        sim.sync()


def test_time_sweep_graph_replays_equal_plain_steps():
    """Once the sweep shape is tuned, fsim_time_sweep replays the step graph
    with event nodes around the sweep: the same kernels in the same order,
    so the state equals that of ordinary steps bit for bit."""
    cfg, pa = cases.make(cases.small_dam_break())
    a = api.Simulation(cfg, pa, device=0)
    b = api.Simulation(cfg, pa, device=0)
    for s in (a, b):
        s.step(4)  # the tuner's step and three graph replays
    tot, sweep = a.time_sweep(5)
    tot2, sweep2 = a.time_sweep(3)  # the captured timed graphs are reused
    b.step(8)
    a.sync()
    b.sync()
    assert 0 < sweep < tot and 0 < sweep2 < tot2
    for f in ("fluid_pos", "fluid_vel", "fluid_rho", "solid_pos", "solid_vel"):
        assert np.array_equal(a.get(f), b.get(f)), f
    a.close()
    b.close()
