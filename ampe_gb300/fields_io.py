"""Initial-condition reader and field writer in NetCDF classic format.

The reference initialises a level from a NetCDF file
(FieldsInitializer::initializeLevelFromData, FieldsInitializer.cc:77-362)
and dumps its fields to one (FieldsWriter.cc:55-489).  Variable names and
layout follow those two: 'phase' (or 'phase0'..'phase2'), optional 'eta'
and 'temperature', 'quat1'..'quat<qlen>' and 'concentration' (one
composition; 'concentration0' is accepted as well) or 'concentration0'..,
each a (z, y, x) array over dimensions 'z', 'y', 'x'; the file's x, y, z
sizes must equal the level's (checkInputFileDimensions,
FieldsInitializer.cc:685-707) and a 2D level takes the file's z slice
`slice_index` (the middle one by default, FieldsInitializer.cc:232-235).
FieldsWriter stores single precision ('f'); float and double variables are
both read.

The container is the classic format (CDF-1, and CDF-2 with 64-bit offsets
for files past 2 GiB), the one the reference reads through its NetCDF-3
code path (HAVE_NETCDF3), implemented here from the published format
description: a big-endian header of dimensions, attributes and variables,
then each non-record variable's data at its recorded offset, padded to four
bytes.  The NETCDF4 (HDF5) container that utils/make_nuclei.py writes by
default is not read: it needs an HDF5 library, which this package does not
carry.
"""
import struct

import numpy as np

_NC_DIMENSION, _NC_VARIABLE, _NC_ATTRIBUTE = 0x0A, 0x0B, 0x0C
_TYPES = {1: np.dtype(">i1"), 2: np.dtype("S1"), 3: np.dtype(">i2"), 4: np.dtype(">i4"),
          5: np.dtype(">f4"), 6: np.dtype(">f8")}
_CODES = {"b": 1, "c": 2, "h": 3, "i": 4, "f": 5, "d": 6}


def _pad(n):
    return (4 - n % 4) % 4


class NetcdfError(ValueError):
    pass


class _Reader:
    def __init__(self, buf):
        self.b = buf
        self.p = 0

    def u32(self):
        v = struct.unpack_from(">I", self.b, self.p)[0]
        self.p += 4
        return v

    def u64(self):
        v = struct.unpack_from(">Q", self.b, self.p)[0]
        self.p += 8
        return v

    def name(self):
        n = self.u32()
        s = bytes(self.b[self.p:self.p + n]).decode("utf-8")
        self.p += n + _pad(n)
        return s

    def values(self, code, n):
        dt = _TYPES.get(code)
        if dt is None:
            raise NetcdfError("unknown NetCDF type %d" % code)
        nb = dt.itemsize * n
        v = np.frombuffer(self.b, dtype=dt, count=n, offset=self.p)
        self.p += nb + _pad(nb)
        return v

    def atts(self):
        tag, n = self.u32(), self.u32()
        if tag == 0 and n == 0:
            return {}
        if tag != _NC_ATTRIBUTE:
            raise NetcdfError("bad attribute list")
        out = {}
        for _ in range(n):
            nm = self.name()
            code, cnt = self.u32(), self.u32()
            v = self.values(code, cnt)
            out[nm] = v.tobytes().decode("utf-8") if code == 2 else v.astype(v.dtype.newbyteorder("="))
        return out


def read(path):
    """A NetCDF classic file as (dims {name: size}, variables {name: array
    in native byte order}, global attributes).  Record variables are not
    supported (the reference writes none)."""
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:3] != b"CDF" or buf[3] not in (1, 2):
        raise NetcdfError("%s: not a NetCDF classic (CDF-1/CDF-2) file" % path)
    wide = buf[3] == 2
    r = _Reader(memoryview(buf))
    r.p = 4
    r.u32()  # number of records
    tag, n = r.u32(), r.u32()
    dims = []
    if not (tag == 0 and n == 0):
        if tag != _NC_DIMENSION:
            raise NetcdfError("bad dimension list")
        for _ in range(n):
            dims.append((r.name(), r.u32()))
    gatts = r.atts()
    tag, n = r.u32(), r.u32()
    variables = {}
    if not (tag == 0 and n == 0):
        if tag != _NC_VARIABLE:
            raise NetcdfError("bad variable list")
        for _ in range(n):
            nm = r.name()
            nd = r.u32()
            ids = [r.u32() for _ in range(nd)]
            r.atts()
            code = r.u32()
            r.u32()  # vsize
            begin = r.u64() if wide else r.u32()
            shape = tuple(dims[i][1] for i in ids)
            if any(s == 0 for s in shape):
                raise NetcdfError("%s: record variable %s not supported" % (path, nm))
            dt = _TYPES[code]
            cnt = int(np.prod(shape)) if shape else 1
            a = np.frombuffer(buf, dtype=dt, count=cnt, offset=begin).reshape(shape)
            variables[nm] = a.astype(dt.newbyteorder("="))
    return dict(dims), variables, gatts


def write(path, variables, dims=None, attributes=None):
    """Write {name: (dimension names, array)} as a NetCDF classic file;
    arrays keep their dtype ('f4', 'f8', 'i4', ...).  dims: {name: size}
    (taken from the arrays when omitted).  CDF-2 when the data pass 2 GiB."""
    dims = dict(dims or {})
    for nm, (dn, a) in variables.items():
        for d, s in zip(dn, np.shape(a)):
            if dims.setdefault(d, s) != s:
                raise NetcdfError("dimension %s: %d and %d" % (d, dims[d], s))
    dnames = list(dims)

    def enc_name(s):
        b = s.encode("utf-8")
        return struct.pack(">I", len(b)) + b + b"\0" * _pad(len(b))

    def enc_atts(atts):
        if not atts:
            return struct.pack(">II", 0, 0)
        out = struct.pack(">II", _NC_ATTRIBUTE, len(atts))
        for k, v in atts.items():
            if isinstance(v, str):
                b = v.encode("utf-8")
                out += enc_name(k) + struct.pack(">II", 2, len(b)) + b + b"\0" * _pad(len(b))
            else:
                v = np.atleast_1d(np.asarray(v))
                code = _CODES[v.dtype.char] if v.dtype.char in _CODES else 6
                vb = v.astype(_TYPES[code]).tobytes()
                out += enc_name(k) + struct.pack(">II", code, v.size) + vb + b"\0" * _pad(len(vb))
        return out

    arrays = []
    for nm, (dn, a) in variables.items():
        a = np.ascontiguousarray(a)
        code = _CODES.get(a.dtype.char)
        if code is None:
            raise NetcdfError("variable %s: dtype %s not storable" % (nm, a.dtype))
        arrays.append((nm, [dnames.index(d) for d in dn], code, a))
    total = sum(a.nbytes + _pad(a.nbytes) for _, _, _, a in arrays)
    wide = total > (1 << 31) - 4096
    head = b"CDF" + bytes([2 if wide else 1]) + struct.pack(">I", 0)
    head += (struct.pack(">II", _NC_DIMENSION, len(dnames)) +
             b"".join(enc_name(d) + struct.pack(">I", dims[d]) for d in dnames)) \
        if dnames else struct.pack(">II", 0, 0)
    head += enc_atts(attributes or {})

    def var_block(offsets):
        out = struct.pack(">II", _NC_VARIABLE, len(arrays)) if arrays else struct.pack(">II", 0, 0)
        for (nm, ids, code, a), off in zip(arrays, offsets):
            vsize = a.nbytes + _pad(a.nbytes)
            out += enc_name(nm) + struct.pack(">I", len(ids)) + \
                b"".join(struct.pack(">I", i) for i in ids) + struct.pack(">II", 0, 0) + \
                struct.pack(">II", code, min(vsize, 0xFFFFFFFF)) + \
                (struct.pack(">Q", off) if wide else struct.pack(">I", off))
        return out

    hlen = len(head) + len(var_block([0] * len(arrays)))
    offsets, off = [], hlen
    for _, _, _, a in arrays:
        offsets.append(off)
        off += a.nbytes + _pad(a.nbytes)
    with open(path, "wb") as f:
        f.write(head + var_block(offsets))
        for _, _, code, a in arrays:
            b = a.astype(_TYPES[code]).tobytes()
            f.write(b + b"\0" * _pad(len(b)))


def read_initial_conditions(path, model, ncompositions=1, slice_index=-1):
    """The fields of `path` for the level of `model`, as the reference's
    FieldsInitializer reads them: returns {'phase', 'concentration' (list),
    and when present 'eta', 'temperature', 'quat' (qlen, z, y, x)}, every
    array float64 with the level's interior shape (z, y, x)."""
    dims, var, _ = read(path)
    nx, ny = model.n[0], model.n[1]
    nz = model.n[2] if model.dim == 3 else 1
    if "phase" not in var:
        raise NetcdfError("could not read variable 'phase' from %s" % path)
    ph = var["phase"]
    if ph.ndim == 2:
        ph = ph[None]
    nz_file, ny_file, nx_file = ph.shape
    if model.dim == 2:
        isl = nz_file // 2 if slice_index < 0 else slice_index
        take = lambda a: (a[None] if a.ndim == 2 else a)[isl:isl + 1]  # noqa: E731
        nz_check = 1
    else:
        take = lambda a: a[None] if a.ndim == 2 else a  # noqa: E731
        nz_check = nz_file
    if (nx_file, ny_file, nz_check) != (nx, ny, nz):
        raise NetcdfError("phase input data dimensions are incorrect: file %d x %d x %d, "
                          "level %d x %d x %d" % (nx_file, ny_file, nz_file, nx, ny, nz))
    out = {"phase": np.ascontiguousarray(take(var["phase"]), dtype=np.float64)}
    for k in ("eta", "temperature"):
        if k in var:
            out[k] = np.ascontiguousarray(take(var[k]), dtype=np.float64)
    conc = []
    for ii in range(ncompositions):
        nm = "concentration%d" % ii if ncompositions > 1 else "concentration"
        if nm not in var and ncompositions == 1:
            nm = "concentration0"
        if nm not in var:
            raise NetcdfError("could not read variable %s from %s" % (nm, path))
        conc.append(np.ascontiguousarray(take(var[nm]), dtype=np.float64))
    out["concentration"] = conc
    q = []
    while "quat%d" % (len(q) + 1) in var:
        q.append(take(var["quat%d" % (len(q) + 1)]))
    if q:
        if "qlen" in dims and dims["qlen"] != len(q):
            raise NetcdfError("qlen %d but %d quaternion components" % (dims["qlen"], len(q)))
        out["quat"] = np.ascontiguousarray(np.stack(q), dtype=np.float64)
    return out


def write_fields(path, phase, concentration=None, quat=None, temperature=None, eta=None,
                 time=None):
    """Dump fields (interior arrays (z, y, x), or (1, y, x) in 2D) as
    FieldsWriter does: single precision, names 'phase', 'eta',
    'quat1'.., 'concentration' (or 'concentration0'.. for several),
    'temperature', dimensions 'x', 'y', 'z' (and 'qlen')."""
    var = {"phase": (("z", "y", "x"), np.asarray(phase, np.float32))}
    if eta is not None:
        var["eta"] = (("z", "y", "x"), np.asarray(eta, np.float32))
    if quat is not None:
        for ii, qc in enumerate(quat):
            var["quat%d" % (ii + 1)] = (("z", "y", "x"), np.asarray(qc, np.float32))
    if concentration is not None:
        cs = concentration if isinstance(concentration, (list, tuple)) else [concentration]
        for ii, c in enumerate(cs):
            nm = "concentration%d" % ii if len(cs) > 1 else "concentration"
            var[nm] = (("z", "y", "x"), np.asarray(c, np.float32))
    if temperature is not None:
        var["temperature"] = (("z", "y", "x"), np.asarray(temperature, np.float32))
    p = np.asarray(phase)
    dims = {"x": p.shape[-1], "y": p.shape[-2], "z": p.shape[-3] if p.ndim == 3 else 1}
    if quat is not None:
        dims["qlen"] = len(quat)
    atts = {"time": float(time)} if time is not None else None
    write(path, var, dims=dims, attributes=atts)
