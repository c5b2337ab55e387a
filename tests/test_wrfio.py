"""History / restart files and the diffwrf comparison (wrf_gb300/wrfio.py).

CPU: the netCDF classic writer and reader round-trip every variable kind;
a history file holds the model's physical domain in WRF's dimension order;
a run restarted from a restart file continues bit for bit (oracle); the
diffwrf statistics follow external/io_netcdf/diffwrf.F90:436-523.
GPU: the same restart continuation on the device, and diffwrf finds no
difference between the GPU's and the oracle's history files."""
import os

import numpy as np
import pytest

from wrf_gb300 import abi, cases, wrfio

from _harness import OracleDomain, STATE_FIELDS, interior, serr


def test_netcdf_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    a = rng.standard_normal((3, 4, 5)).astype(np.float32)
    b = rng.standard_normal((3, 7)).astype(np.float64)
    c = np.arange(6, dtype=np.int32).reshape(2, 3)
    t = np.frombuffer(b"0001-01-01_00:00:000001-01-01_00:00:010001-01-01_00:00:02", dtype="S1").reshape(3, 19)
    dims = [("Time", None), ("x", 5), ("y", 4), ("z", 7), ("p", 2), ("q", 3), ("DateStrLen", 19)]
    var = [("Times", ("Time", "DateStrLen"), wrfio.NC_CHAR, {}, t),
           ("A", ("Time", "y", "x"), wrfio.NC_FLOAT, {"units": "m", "FieldType": 104}, a),
           ("B", ("Time", "z"), wrfio.NC_DOUBLE, {}, b),
           ("C", ("p", "q"), wrfio.NC_INT, {"scale": np.float32(2.5)}, c)]
    p = str(tmp_path / "x.nc")
    wrfio.write_netcdf(p, dims, var, {"TITLE": "t", "DX": np.float32(2000.0), "N": 3}, 3)
    assert open(p, "rb").read(4) == b"CDF\x02"
    d, g, v = wrfio.read_netcdf(p)
    assert dict(d)["Time"] == 0 and dict(d)["x"] == 5
    assert g["TITLE"] == "t" and float(g["DX"][0]) == 2000.0 and int(g["N"][0]) == 3
    assert np.array_equal(v["A"][2], a) and v["A"][1]["units"] == "m" and int(v["A"][1]["FieldType"][0]) == 104
    assert np.array_equal(v["B"][2], b) and np.array_equal(v["C"][2], c)
    assert v["Times"][2].tobytes() == t.tobytes()


def test_wrfout_layout(tmp_path):
    case = cases.small_case(nx=16, ny=12, kde=14, n_scalar=1, seed=5)
    od = OracleDomain(case, "f32")
    od.step(1)
    p = str(tmp_path / "wrfout_d01")
    wrfio.write_wrfout(p, case.desc, [od.get])
    _, g, v = wrfio.read_netcdf(p)
    assert int(g["WEST-EAST_GRID_DIMENSION"][0]) == case.ide
    dn, atts, u = v["U"]
    assert dn == ["Time", "bottom_top", "south_north", "west_east_stag"] and atts["stagger"] == "X"
    assert u.shape == (1, case.kde - 1, case.jde - 1, case.ide)
    h = abi.HALO
    mem = od.get(abi.FIELD_ID["u_2"]).reshape(case.jde + 2 * h, case.kde, -1)
    # U(Time, k, j, i) is the Fortran u(i, k, j) of the physical domain
    assert u[0, 3, 5, 7] == np.float32(mem[h + 5, 3, h + 7])
    assert v["W"][2].shape == (1, case.kde, case.jde - 1, case.ide - 1)
    assert v["MU"][2].shape == (1, case.jde - 1, case.ide - 1)
    assert v["QVAPOR"][2].shape == (1, case.kde - 1, case.jde - 1, case.ide - 1)


def _restart_case():
    return cases.small_case(nx=16, ny=12, kde=14, n_scalar=2, seed=8)


def test_restart_continues_bitwise_oracle(tmp_path):
    """2 steps, restart file, a fresh domain loaded from it and 2 more steps:
    every state field and species bit for bit the uninterrupted 4 steps."""
    case = _restart_case()
    od = OracleDomain(case, "f32")
    od.step(2)
    p = str(tmp_path / "wrfrst_d01")
    wrfio.write_wrfrst(p, case.desc, od.get)
    od.step(2)
    od2 = OracleDomain(case, "f32", load=False)
    wrfio.read_wrfrst(p, case.desc, lambda f, a: od2.set(f, a), od2.fill_halo)
    od2.step(2)
    nsp = case.desc.n_moist + case.desc.n_scalar
    ids = [abi.FIELD_ID[n] for n in STATE_FIELDS] + [abi.species_id(s) for s in range(nsp)]
    for fid in ids:
        assert np.array_equal(interior(case, fid, od.get(fid)), interior(case, fid, od2.get(fid))), fid


def test_diffwrf_statistics(tmp_path):
    case = cases.small_case(nx=16, ny=12, kde=14, n_scalar=1, seed=5)
    od = OracleDomain(case, "f32")
    od.step(1)
    p1, p2 = str(tmp_path / "a"), str(tmp_path / "b")
    wrfio.write_wrfout(p1, case.desc, [od.get])
    wrfio.write_wrfout(p2, case.desc, [od.get])
    lines = []
    res = wrfio.diffwrf(p1, p2, out=lines.append)
    assert not lines and all(s["ndifs"] == 0 and s["digits"] == 15 for s in res.values())
    # perturb theta in one file: diffwrf reports it with the harness's serr
    fid = abi.FIELD_ID["t_2"]
    h = abi.HALO
    t = od.get(fid).copy()
    t.reshape(case.jde + 2 * h, case.kde, -1)[h + 4, 5, h + 6] += 0.5  # a physical-domain point
    wrfio.write_wrfout(p2, case.desc, [lambda f: t if f == fid else od.get(f)])
    res = wrfio.diffwrf(p1, p2, out=lines.append)
    st = res[(0, "THM")]
    assert st["ndifs"] == 1 and len(lines) >= 2 and "THM" in lines[1]
    a = wrfio.read_netcdf(p1)[2]["THM"][2]
    b = wrfio.read_netcdf(p2)[2]["THM"][2]
    assert abs(st["serr"] - serr(a, b)) <= 1e-15
    assert st["perr"] == pytest.approx(0.5 / float(np.max(np.abs(b))), rel=1e-6)


@pytest.mark.gpu
def test_restart_continues_bitwise_gpu(gpulib, tmp_path):
    """The device domain: restart file after 2 steps, a fresh domain loaded
    from it, 2 more steps: bit for bit the uninterrupted run; and diffwrf
    finds no difference between the GPU's and the oracle's history files."""
    from wrf_gb300 import gpu as G
    case = _restart_case()
    a = G.Domain(case)
    a.step(2)
    a.sync()
    p = str(tmp_path / "wrfrst_d01")
    wrfio.write_wrfrst(p, case.desc, lambda f: a.get(0, f))
    a.step(2)
    a.sync()
    b = G.Domain(case)
    wrfio.read_wrfrst(p, case.desc, lambda f, arr: b.set(0, f, arr), b.fill_halo)
    b.step(2)
    b.sync()
    nsp = case.desc.n_moist + case.desc.n_scalar
    ids = [abi.FIELD_ID[n] for n in STATE_FIELDS] + [abi.species_id(s) for s in range(nsp)]
    for fid in ids:
        assert np.array_equal(interior(case, fid, a.get(0, fid)), interior(case, fid, b.get(0, fid))), fid
    od = OracleDomain(case, "f32")
    od.step(4)
    pg, po = str(tmp_path / "wrfout_gpu"), str(tmp_path / "wrfout_oracle")
    wrfio.write_wrfout(pg, case.desc, [lambda f: a.get(0, f)])
    wrfio.write_wrfout(po, case.desc, [od.get])
    lines = []
    res = wrfio.diffwrf(pg, po, out=lines.append)
    assert not lines, lines
    assert all(s["ndifs"] == 0 for s in res.values())
