"""WRF history / restart files and the diffwrf comparison, without a netCDF
library.

The reference writes its history (wrfout) and restart (wrfrst) files through
its I/O API into netCDF (share/output_wrf.F, share/wrf_restartout.F,
external/io_netcdf/wrf_io.F90), and compares two such files with diffwrf
(external/io_netcdf/diffwrf.F90).  This module reads and writes the netCDF
classic format (the 64-bit-offset variant, "CDF-2") directly with numpy, so
files written here open in any netCDF tool and files from such tools open
here, and it restates diffwrf's per-field statistics.

Layout: the WRF conventions of those files.  Every field is a record
variable along the unlimited dimension Time; 3-D fields are (Time,
bottom_top[_stag], south_north[_stag], west_east[_stag]) in C order, which
is the model's (i, j, k) Fortran order; each carries FieldType (104 for
REAL), MemoryOrder ("XYZ", "XY", "Z", "0"), description, units and stagger
("X", "Y", "Z" or "").  Only the physical domain is stored (no halo), as the
reference does; a restart read back fills the halos with the domain's own
boundary fill.

Names follow the Registry (Registry.EM_COMMON): U, V, W, PH, PHB, T (dry
potential temperature perturbation), THM (the prognostic moist one,
use_theta_m = 1), MU, MUB, P, PB, AL, ALB, QVAPOR; a restart adds the two
time levels (U_1, U_2, ..., MU_1, MU_2) and every other array the step
carries, so that a run restarted from it continues bit for bit.
"""
import struct

import numpy as np

from . import abi

NC_BYTE, NC_CHAR, NC_SHORT, NC_INT, NC_FLOAT, NC_DOUBLE = 1, 2, 3, 4, 5, 6
_NC_DIMENSION, _NC_VARIABLE, _NC_ATTRIBUTE = 10, 11, 12
_DTYPE = {NC_BYTE: ">i1", NC_CHAR: "S1", NC_SHORT: ">i2", NC_INT: ">i4", NC_FLOAT: ">f4", NC_DOUBLE: ">f8"}
_SIZE = {NC_BYTE: 1, NC_CHAR: 1, NC_SHORT: 2, NC_INT: 4, NC_FLOAT: 4, NC_DOUBLE: 8}
WRF_REAL = 104  # FieldType of REAL fields (frame/module_io.F)


def _pad4(n):
    return (n + 3) & ~3


class _Writer:
    def __init__(self):
        self.b = bytearray()

    def i32(self, v):
        self.b += struct.pack(">i", v)

    def i64(self, v):
        self.b += struct.pack(">q", v)

    def name(self, s):
        raw = s.encode()
        self.i32(len(raw))
        self.b += raw + b"\0" * (_pad4(len(raw)) - len(raw))

    def values(self, nctype, data):
        raw = np.ascontiguousarray(data, dtype=_DTYPE[nctype]).tobytes() if nctype != NC_CHAR else data
        self.b += raw + b"\0" * (_pad4(len(raw)) - len(raw))


def _att_value(v):
    if isinstance(v, str):
        return NC_CHAR, v.encode(), len(v.encode())
    if isinstance(v, (bool, int, np.integer)):
        return NC_INT, np.array([v]), 1
    a = np.atleast_1d(np.asarray(v))
    if a.dtype.kind in "iu":
        return NC_INT, a, a.size
    if a.dtype == np.float64:
        return NC_DOUBLE, a, a.size
    return NC_FLOAT, a.astype(np.float32), a.size


def _write_atts(w, atts):
    if not atts:
        w.i32(0); w.i32(0)
        return
    w.i32(_NC_ATTRIBUTE); w.i32(len(atts))
    for k, v in atts.items():
        t, data, n = _att_value(v)
        w.name(k); w.i32(t); w.i32(n); w.values(t, data)


def write_netcdf(path, dims, variables, gatts, nrec):
    """Write a CDF-2 file.  dims: [(name, length)] with length None for the
    unlimited (record) dimension; variables: [(name, dim names, nc type,
    attributes, data)] where data's leading axis is the record axis for
    record variables."""
    dim_index = {d[0]: q for q, d in enumerate(dims)}
    rec_dim = [d[0] for d in dims if d[1] is None]
    rec_dim = rec_dim[0] if rec_dim else None

    def shape_of(dnames):
        return [nrec if dn == rec_dim else dict(dims)[dn] for dn in dnames]

    # vsize of every variable (one record's slab for record variables)
    info = []
    for name, dnames, t, atts, data in variables:
        is_rec = bool(dnames) and dnames[0] == rec_dim
        n = int(np.prod(shape_of(dnames)[1:] if is_rec else shape_of(dnames)))
        info.append((is_rec, _pad4(n * _SIZE[t]), n * _SIZE[t]))
    rec_vars = [q for q, x in enumerate(info) if x[0]]
    # the one-record-variable special case of the format: no padding
    recsize = info[rec_vars[0]][2] if len(rec_vars) == 1 else sum(info[q][1] for q in rec_vars)

    def header(begins):
        w = _Writer()
        w.b += b"CDF\x02"
        w.i32(nrec)
        w.i32(_NC_DIMENSION); w.i32(len(dims))
        for dn, ln in dims:
            w.name(dn); w.i32(0 if ln is None else ln)
        _write_atts(w, gatts)
        w.i32(_NC_VARIABLE); w.i32(len(variables))
        for q, (name, dnames, t, atts, data) in enumerate(variables):
            w.name(name); w.i32(len(dnames))
            for dn in dnames:
                w.i32(dim_index[dn])
            _write_atts(w, atts)
            w.i32(t); w.i32(min(info[q][1], 2 ** 32 - 4)); w.i64(begins[q])
        return w.b

    hlen = len(header([0] * len(variables)))
    begins, off = [0] * len(variables), hlen
    for q, x in enumerate(info):
        if not x[0]:
            begins[q] = off
            off += x[1]
    rec_start = off
    for q in rec_vars:
        begins[q] = off
        off += info[q][1] if len(rec_vars) > 1 else info[q][2]
    with open(path, "wb") as f:
        f.write(header(begins))
        for q, (name, dnames, t, atts, data) in enumerate(variables):
            if info[q][0]:
                continue
            raw = np.ascontiguousarray(data, dtype=_DTYPE[t]).tobytes() if t != NC_CHAR else bytes(data)
            f.write(raw + b"\0" * (info[q][1] - len(raw)))
        for r in range(nrec):
            assert f.tell() == rec_start + r * recsize
            for q in rec_vars:
                name, dnames, t, atts, data = variables[q]
                slab = data[r]
                raw = np.ascontiguousarray(slab, dtype=_DTYPE[t]).tobytes() if t != NC_CHAR else bytes(slab)
                pad = (info[q][1] if len(rec_vars) > 1 else info[q][2]) - len(raw)
                f.write(raw + b"\0" * pad)


def read_netcdf(path):
    """Read a netCDF classic file (CDF-1 or CDF-2): returns (dims, global
    attributes, {name: (dim names, attributes, array)})."""
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:3] != b"CDF" or buf[3] not in (1, 2):
        raise ValueError("%s: not a netCDF classic file" % path)
    off64 = buf[3] == 2
    pos = [4]

    def i32():
        v = struct.unpack_from(">i", buf, pos[0])[0]
        pos[0] += 4
        return v

    def name():
        n = i32()
        s = buf[pos[0]:pos[0] + n].decode()
        pos[0] += _pad4(n)
        return s

    def atts():
        tag, n = i32(), i32()
        out = {}
        for _ in range(n if tag == _NC_ATTRIBUTE else 0):
            k = name()
            t, cnt = i32(), i32()
            raw = buf[pos[0]:pos[0] + cnt * _SIZE[t]]
            pos[0] += _pad4(cnt * _SIZE[t])
            out[k] = raw.decode() if t == NC_CHAR else np.frombuffer(raw, dtype=_DTYPE[t]).copy()
        return out

    nrec = i32()
    tag, ndim = i32(), i32()
    dims = []
    for _ in range(ndim if tag == _NC_DIMENSION else 0):
        dn = name()
        dims.append((dn, i32()))
    gatts = atts()
    tag, nvar = i32(), i32()
    vars_ = []
    for _ in range(nvar if tag == _NC_VARIABLE else 0):
        vn = name()
        nd = i32()
        dids = [i32() for _ in range(nd)]
        va = atts()
        t, vsize = i32(), i32()
        if off64:
            begin = struct.unpack_from(">q", buf, pos[0])[0]
            pos[0] += 8
        else:
            begin = i32()
        vars_.append((vn, dids, va, t, vsize, begin))
    rec_vars = [v for v in vars_ if v[1] and dims[v[1][0]][1] == 0]
    recsize = sum(v[4] for v in rec_vars) if len(rec_vars) > 1 else (
        int(np.prod([dims[d][1] for d in rec_vars[0][1][1:]])) * _SIZE[rec_vars[0][3]] if rec_vars else 0)
    out = {}
    for vn, dids, va, t, vsize, begin in vars_:
        dnames = [dims[d][0] for d in dids]
        is_rec = bool(dids) and dims[dids[0]][1] == 0
        shp = [dims[d][1] for d in dids[1:]] if is_rec else [dims[d][1] for d in dids]
        n = int(np.prod(shp)) if shp else 1
        if is_rec:
            recs = [np.frombuffer(buf, dtype=_DTYPE[t], count=n, offset=begin + r * recsize).reshape(shp)
                    for r in range(nrec)]
            arr = np.stack(recs) if recs else np.zeros([0] + shp, dtype=_DTYPE[t])
        else:
            arr = np.frombuffer(buf, dtype=_DTYPE[t], count=n, offset=begin).reshape(shp)
        out[vn] = (dnames, va, np.array(arr))
    return dims, gatts, out


# ---------------------------------------------------------------------------
# WRF field conventions
# ---------------------------------------------------------------------------
# name in the file -> (field id name, stagger, description, units)
_F3 = {
    "U": ("u_2", "X", "x-wind component", "m s-1"),
    "V": ("v_2", "Y", "y-wind component", "m s-1"),
    "W": ("w_2", "Z", "z-wind component", "m s-1"),
    "PH": ("ph_2", "Z", "perturbation geopotential", "m2 s-2"),
    "PHB": ("phb", "Z", "base-state geopotential", "m2 s-2"),
    "THM": ("t_2", "", "perturbation moist potential temperature (1+Rv/Rd Qv)(theta)-T0", "K"),
    "P": ("p", "", "perturbation pressure", "Pa"),
    "PB": ("pb", "", "BASE STATE PRESSURE", "Pa"),
    "AL": ("al", "", "inverse perturbation density", "m3 kg-1"),
    "ALB": ("alb", "", "inverse base density", "m3 kg-1"),
}
_F2 = {
    "MU": ("mu_2", "perturbation dry air mass in column", "Pa"),
    "MUB": ("mub", "base state dry air mass in column", "Pa"),
    "HGT": ("ht", "Terrain Height", "m"),
    "MAPFAC_MX": ("msftx", "Map scale factor on mass grid, x direction", ""),
    "MAPFAC_MY": ("msfty", "Map scale factor on mass grid, y direction", ""),
    "F": ("f", "Coriolis sine latitude term", "s-1"),
    "E": ("e", "Coriolis cosine latitude term", "s-1"),
    "SINALPHA": ("sina", "Local sine of map rotation", ""),
    "COSALPHA": ("cosa", "Local cosine of map rotation", ""),
}
_F1 = {"ZNU": "znu", "ZNW": "znw", "DNW": "dnw", "RDNW": "rdnw", "DN": "dn", "RDN": "rdn", "FNM": "fnm",
       "FNP": "fnp", "C1H": "c1h", "C2H": "c2h", "C1F": "c1f", "C2F": "c2f", "C3H": "c3h", "C4H": "c4h",
       "C3F": "c3f", "C4F": "c4f"}
_RV_RD = 461.6 / 287.0


def _stag_of(fid):
    """Stagger of a state field: 'X', 'Y', 'Z' or ''."""
    nm = [k for k, v in abi.FIELD_ID.items() if v == fid]
    nm = nm[0] if nm else ""
    if nm.startswith("u_") or nm in ("ru", "ru_m", "ru_tend", "u_save", "cqu"):
        return "X"
    if nm.startswith("v_") or nm in ("rv", "rv_m", "rv_tend", "v_save", "cqv"):
        return "Y"
    if nm.startswith("w_") or nm.startswith("ph") or nm in ("rw", "ww", "ww1", "ww_m", "rw_tend", "w_save",
                                                              "cqw", "php", "a", "alpha", "gamma"):
        return "Z"
    return ""


def _interior3(arr, ide, jde, kde, stag):
    """(jms:jme, kms:kme, ims:ime) memory array -> (k, j, i) physical domain."""
    h = abi.HALO
    a = np.asarray(arr).reshape(jde + 2 * h, kde, -1)
    ni = ide if stag == "X" else ide - 1
    nj = jde if stag == "Y" else jde - 1
    nk = kde if stag == "Z" else kde - 1
    return np.ascontiguousarray(a[h:h + nj, :nk, h:h + ni].transpose(1, 0, 2))


def _interior2(arr, ide, jde):
    h = abi.HALO
    a = np.asarray(arr).reshape(jde + 2 * h, -1)
    return np.ascontiguousarray(a[h:h + jde - 1, h:h + ide - 1])


def _dimnames(stag, nd):
    if nd == 2:
        return ("Time", "south_north", "west_east")
    return ("Time", "bottom_top_stag" if stag == "Z" else "bottom_top",
            "south_north_stag" if stag == "Y" else "south_north",
            "west_east_stag" if stag == "X" else "west_east")


def _gatts(desc, title):
    c = desc.config
    s = desc.scalars
    return {"TITLE": title, "START_DATE": "0001-01-01_00:00:00",
            "WEST-EAST_GRID_DIMENSION": int(desc.ide), "SOUTH-NORTH_GRID_DIMENSION": int(desc.jde),
            "BOTTOM-TOP_GRID_DIMENSION": int(desc.kde), "DX": np.float32(s.dx), "DY": np.float32(s.dy),
            "DT": np.float32(s.dt), "P_TOP": np.float32(s.p_top), "HYPSOMETRIC_OPT": int(c.hypsometric_opt),
            "USE_THETA_M": int(c.use_theta_m), "MOIST_ADV_OPT": int(c.moist_adv_opt),
            "SCALAR_ADV_OPT": int(c.scalar_adv_opt), "DIFF_6TH_OPT": int(c.diff_6th_opt),
            "DAMP_OPT": int(c.damp_opt), "W_DAMPING": int(c.w_damping), "NUM_MOIST": int(desc.n_moist),
            "NUM_SCALAR": int(desc.n_scalar), "PERIODIC_X": int(c.periodic_x), "PERIODIC_Y": int(c.periodic_y),
            "SYMMETRIC_YS": int(c.symmetric_ys), "SYMMETRIC_YE": int(c.symmetric_ye)}


def _dims(desc):
    return [("Time", None), ("DateStrLen", 19), ("west_east", desc.ide - 1), ("south_north", desc.jde - 1),
            ("bottom_top", desc.kde - 1), ("west_east_stag", desc.ide), ("south_north_stag", desc.jde),
            ("bottom_top_stag", desc.kde)]


def _var(name, dnames, data, desc_, units, stagger, order):
    atts = {"FieldType": WRF_REAL, "MemoryOrder": order, "description": desc_, "units": units,
            "stagger": stagger}
    return (name, dnames, NC_FLOAT, atts, np.asarray(data, dtype=np.float32))


def _times(frames):
    return np.frombuffer("".join(t.ljust(19)[:19] for t in frames).encode(), dtype="S1").reshape(len(frames), 19)


def write_wrfout(path, desc, frames, times=None, title="OUTPUT FROM WRF-GB300 (WRF-ARW dynamics)"):
    """History file of one domain: frames is a list of getters get(fid) ->
    memory-layout array (one per output time).  Fields: U, V, W, PH, PHB, T,
    THM, MU, MUB, P, PB, QVAPOR, the passive scalars TR01.., the eta and
    hybrid metrics and the 2-D map/Coriolis fields."""
    ide, jde, kde = desc.ide, desc.jde, desc.kde
    nsp = desc.n_moist + desc.n_scalar
    times = times or ["0001-01-01_00:00:%02d" % q for q in range(len(frames))]
    var = [("Times", ("Time", "DateStrLen"), NC_CHAR, {}, _times(times))]
    for nm in ("U", "V", "W", "PH", "PHB", "THM", "P", "PB"):
        fid_nm, st, d, u = _F3[nm]
        fid = abi.FIELD_ID[fid_nm]
        data = np.stack([_interior3(g(fid), ide, jde, kde, st) for g in frames])
        var.append(_var(nm, _dimnames(st, 3), data, d, u, st, "XYZ"))
    # dry potential temperature perturbation from the moist one (use_theta_m = 1)
    thm = np.stack([_interior3(g(abi.FIELD_ID["t_2"]), ide, jde, kde, "") for g in frames]).astype(np.float32)
    qv = np.stack([_interior3(g(abi.species_id(0)), ide, jde, kde, "") for g in frames]).astype(np.float32)
    t = (thm + np.float32(300.0)) / (np.float32(1.0) + np.float32(_RV_RD) * qv) - np.float32(300.0)
    var.append(_var("T", _dimnames("", 3), t, "perturbation potential temperature theta-t0", "K", "", "XYZ"))
    var.append(_var("QVAPOR", _dimnames("", 3), qv, "Water vapor mixing ratio", "kg kg-1", "", "XYZ"))
    for s in range(1, nsp):
        data = np.stack([_interior3(g(abi.species_id(s)), ide, jde, kde, "") for g in frames])
        var.append(_var("TR%02d" % s, _dimnames("", 3), data, "passive scalar %d" % s, "kg kg-1", "", "XYZ"))
    for nm, (fid_nm, d, u) in _F2.items():
        fid = abi.FIELD_ID[fid_nm]
        data = np.stack([_interior2(g(fid), ide, jde) for g in frames])
        var.append(_var(nm, _dimnames("", 2), data, d, u, "", "XY"))
    for nm, fid_nm in _F1.items():
        fid = abi.FIELD_ID[fid_nm]
        stag = nm in ("ZNW", "C3F", "C4F", "C1F", "C2F", "DN", "RDN", "FNM", "FNP")
        n = kde if stag else kde - 1
        data = np.stack([np.asarray(g(fid))[:n] for g in frames])
        var.append(_var(nm, ("Time", "bottom_top_stag" if stag else "bottom_top"), data, nm.lower(), "",
                        "Z" if stag else "", "Z"))
    var.append(_var("P_TOP", ("Time",), np.full(len(frames), desc.scalars.p_top), "PRESSURE TOP OF THE MODEL",
                    "Pa", "", "0"))
    write_netcdf(path, _dims(desc), var, _gatts(desc, title), len(frames))


def _restart_fields(desc):
    """(file name, field id, stagger, kind) of every array of a restart."""
    out = []
    for nm, fid in abi.FIELD_ID.items():
        if nm in abi.TENDF:  # stage 1's forward tendencies: rebuilt at every step's first stage
            continue
        k = abi.field_kind(fid)
        out.append((nm.upper(), fid, _stag_of(fid) if k == 3 else "", k))
    nsp = desc.n_moist + desc.n_scalar
    for s in range(nsp):
        base = "QVAPOR" if s == 0 else "TR%02d" % s
        out.append((base + "_2", abi.species_id(s), "", 3))
        out.append((base + "_1", abi.species_id(s, True), "", 3))
    return out


def write_wrfrst(path, desc, get, time="0001-01-01_00:00:00", title="RESTART FROM WRF-GB300 (WRF-ARW dynamics)"):
    """Restart file of one domain at one time: every array of the field
    table (both time levels, base state, metrics, the step's carried
    diagnostics) and every species, current (_2) and old (_1).  get(fid)
    returns the memory-layout array."""
    ide, jde, kde = desc.ide, desc.jde, desc.kde
    var = [("Times", ("Time", "DateStrLen"), NC_CHAR, {}, _times([time]))]
    for nm, fid, st, k in _restart_fields(desc):
        if k == 3:
            data = _interior3(get(fid), ide, jde, kde, st)[None]
            var.append(_var(nm, _dimnames(st, 3), data, nm.lower(), "", st, "XYZ"))
        elif k == 2:
            var.append(_var(nm, _dimnames("", 2), _interior2(get(fid), ide, jde)[None], nm.lower(), "", "", "XY"))
        else:
            var.append(_var(nm, ("Time", "bottom_top_stag"), np.asarray(get(fid))[None, :kde], nm.lower(), "", "Z",
                            "Z"))
    write_netcdf(path, _dims(desc), var, _gatts(desc, title), 1)


def read_wrfrst(path, desc, set_field, fill_halo):
    """Load a restart written by write_wrfrst into a domain of the same
    description: set_field(fid, memory-layout array) for every array, then
    fill_halo(fid, var) of every 3-D and 2-D field with its stagger (the
    periodic / symmetric boundary fill), as a restarted reference run fills
    its halos before the first step."""
    dims, gatts, vars_ = read_netcdf(path)
    if (int(gatts["WEST-EAST_GRID_DIMENSION"][0]), int(gatts["SOUTH-NORTH_GRID_DIMENSION"][0]),
            int(gatts["BOTTOM-TOP_GRID_DIMENSION"][0])) != (desc.ide, desc.jde, desc.kde):
        raise ValueError("%s: domain dimensions differ from the description" % path)
    h = abi.HALO
    ide, jde, kde = desc.ide, desc.jde, desc.kde
    var_of = {"X": "u", "Y": "v", "Z": "w", "": "p"}
    for nm, fid, st, k in _restart_fields(desc):
        data = vars_[nm][2][0].astype(np.float32)
        if k == 3:
            a = np.zeros((jde + 2 * h, kde, ide + 2 * h), np.float32)
            nk, nj, ni = data.shape
            a[h:h + nj, :nk, h:h + ni] = data.transpose(1, 0, 2)
            set_field(fid, a)
            fill_halo(fid, var_of[st])
        elif k == 2:
            a = np.zeros((jde + 2 * h, ide + 2 * h), np.float32)
            a[h:h + jde - 1, h:h + ide - 1] = data
            set_field(fid, a)
            fill_halo(fid, "t")
        else:
            set_field(fid, data[:kde])


# ---------------------------------------------------------------------------
# diffwrf
# ---------------------------------------------------------------------------
def field_stats(a, b):
    """diffwrf's statistics of one field (external/io_netcdf/diffwrf.F90:
    436-523), in double precision over every point: number of differing
    points, RMS of each, digits of agreement of the RMS, RMSE, the
    point-wise max |a-b| / max |b| (perr) and the relative L2 error serr."""
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    n = a.size
    sume = float(np.sum((a - b) * (a - b)))
    sum1 = float(np.sum(a * a))
    sum2 = float(np.sum(b * b))
    diff1 = float(np.max(np.abs(a - b))) if n else 0.0
    diff2 = float(np.max(np.abs(b))) if n else 0.0
    ndif = int(np.count_nonzero(a != b))
    rmse = (sume / n) ** 0.5 if n else 0.0
    rms1 = (sum1 / n) ** 0.5 if n else 0.0
    rms2 = (sum2 / n) ** 0.5 if n else 0.0
    serr = (sume / sum2) ** 0.5 if sum2 > 0.0 else (1.0 if sume > 0.0 else 0.0)
    perr = diff1 / diff2 if diff2 > 0.0 else (1.0 if diff1 > 0.0 else 0.0)
    digits = 0
    if rms1 - rms2 == 0.0:
        digits = 15
    elif rms2 != 0.0:
        tmp1 = 1.0 / (abs(rms1 - rms2) / rms2)
        if tmp1 != 0.0:
            digits = int(np.log10(tmp1))  # Fortran assigns the real to an INTEGER: truncation
    return {"ndifs": ndif, "rms1": rms1, "rms2": rms2, "digits": digits, "rmse": rmse, "perr": perr,
            "serr": serr}


def diffwrf(path1, path2, out=print):
    """Compare every REAL field the two files share, time by time, and print
    the fields that differ in diffwrf's table format; returns
    {(time index, field): statistics}."""
    _, _, v1 = read_netcdf(path1)
    _, _, v2 = read_netcdf(path2)
    res = {}
    header_done = False
    nt = min(v1["Times"][2].shape[0], v2["Times"][2].shape[0]) if "Times" in v1 and "Times" in v2 else 1
    for t in range(nt):
        for nm, (dn, atts, a) in v1.items():
            if nm == "Times" or nm not in v2 or a.dtype.kind != "f":
                continue
            b = v2[nm][2]
            if a.shape != b.shape:
                out(" Big difference: dim lengths differ for %s" % nm)
                continue
            st = field_stats(a[t], b[t])
            res[(t, nm)] = st
            if st["ndifs"]:
                if not header_done:
                    out("     Field   Ndifs    Dims       RMS (1)            RMS (2)     DIGITS    RMSE     "
                        "pntwise max")
                    header_done = True
                ndim = a.ndim - 1
                out("%10s %9d  %3d %18.10E %18.10E %3d %12.4E %12.4E" % (
                    nm[:10], st["ndifs"], ndim, st["rms1"], st["rms2"], st["digits"], st["rmse"], st["perr"]))
    return res


def main(argv=None):
    import sys
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 2:
        print("usage: python -m wrf_gb300.wrfio FILE1 FILE2   (diffwrf-style comparison)")
        return 2
    diffwrf(argv[0], argv[1])
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
