"""BraWl's netCDF outputs and inputs without libnetcdf: a writer and reader
of the classic format (CDF-1) for the files the sampling path produces.

* configurations   -- ncdf_grid_state_writer / ncdf_config_reader
                      (src/netcdf_io.f90:495-583, 1368-1429): variable
                      "configuration" (NC_SHORT) over dims b, x, y, z and the
                      global attributes N_basis, N_1, N_2, N_3, Number of
                      Species, Lattice Type, Concentrations.
* radial densities -- ncdf_radial_density_writer / _reader (:150-244,
                      :1443-1516): "rho data" over i, j, r, T, then
                      "r data", "T data", "U data", with the run's global
                      attributes plus Interaction file and Warren-Cowley
                      Range.
* 1-D data         -- ncdf_writer_1d (:731-806): "grid data" over x (the
                      Wang-Landau density of states).
* ALRO             -- ncdf_order_writer (:362-480): "grid data" holding
                      order(species, basis, x, y, z, T) under the dimension
                      names the reference gives it (b, x, y, z, s, t, in
                      that order), and "temperature data" over temp.

The layout is the one the netCDF library gives a file created with
NF90_CLOBBER and closed after one enddef: header, then each variable's data
in definition order, every section padded to 4 bytes, big-endian values.
Files written here are byte-for-byte those of the reference for the same
data (the golden test outputs are compared byte by byte).  Fortran's
column-major (b, x, y, z) is the C-ordered (z, y, x, b) array stored.
"""
from __future__ import annotations

import struct

import numpy as np

__all__ = ["write_config", "read_config", "write_radial_density", "read_radial_density",
           "write_grid_1d", "write_order", "read_file"]

_MAGIC = b"CDF\x01"
_ABSENT = b"\x00" * 8
_NC_DIMENSION, _NC_VARIABLE, _NC_ATTRIBUTE = 0x0A, 0x0B, 0x0C
# nc_type codes and their big-endian element types
_TYPES = {1: ">i1", 2: "S1", 3: ">i2", 4: ">i4", 5: ">f4", 6: ">f8"}
_CODES = {np.dtype(">i1"): 1, np.dtype(">i2"): 3, np.dtype(">i4"): 4, np.dtype(">f4"): 5,
          np.dtype(">f8"): 6}


def _pad4(b: bytes) -> bytes:
    return b + b"\x00" * (-len(b) % 4)


def _name(s: str) -> bytes:
    raw = s.encode()
    return struct.pack(">i", len(raw)) + _pad4(raw)


def _attr_value(v):
    """(nc_type, nelems, payload) of a global attribute value."""
    if isinstance(v, (str, bytes)):
        raw = v.encode() if isinstance(v, str) else v
        return 2, len(raw), _pad4(raw)
    a = np.asarray(v)
    if a.dtype.kind in "iu":
        a = a.astype(">i4")
    elif a.dtype.kind == "f":
        a = a.astype(">f8")
    else:
        raise TypeError(f"unsupported attribute type {a.dtype}")
    a = a.ravel()
    return _CODES[a.dtype], a.size, _pad4(a.tobytes())


def _encode(dims, attrs, variables) -> bytes:
    """dims: [(name, length)]; attrs: [(name, value)]; variables:
    [(name, [dim names], big-endian ndarray)] in definition order."""
    dim_index = {n: i for i, (n, _) in enumerate(dims)}
    out = [_MAGIC, struct.pack(">i", 0)]
    if dims:
        out.append(struct.pack(">ii", _NC_DIMENSION, len(dims)))
        for n, length in dims:
            out.append(_name(n) + struct.pack(">i", length))
    else:
        out.append(_ABSENT)
    if attrs:
        out.append(struct.pack(">ii", _NC_ATTRIBUTE, len(attrs)))
        for n, v in attrs:
            code, nelems, payload = _attr_value(v)
            out.append(_name(n) + struct.pack(">ii", code, nelems) + payload)
    else:
        out.append(_ABSENT)
    # the header's size does not depend on the begin offsets (4 bytes each)
    var_heads = []
    for n, dnames, data in variables:
        h = _name(n) + struct.pack(">i", len(dnames))
        h += b"".join(struct.pack(">i", dim_index[d]) for d in dnames)
        h += _ABSENT  # no variable attributes
        vsize = data.nbytes + (-data.nbytes % 4)
        h += struct.pack(">ii", _CODES[data.dtype], vsize)
        var_heads.append((h, vsize))
    if variables:
        out.append(struct.pack(">ii", _NC_VARIABLE, len(variables)))
    else:
        out.append(_ABSENT)
    header_len = sum(len(b) for b in out) + sum(len(h) + 4 for h, _ in var_heads)
    begin = header_len
    for h, vsize in var_heads:
        out.append(h + struct.pack(">i", begin))
        begin += vsize
    for _, _, data in variables:
        out.append(_pad4(data.tobytes()))
    return b"".join(out)


def _read_name(buf, off):
    (n,) = struct.unpack_from(">i", buf, off)
    off += 4
    s = bytes(buf[off:off + n]).decode()
    return s, off + n + (-n % 4)


def _read_attrs(buf, off):
    tag, count = struct.unpack_from(">ii", buf, off)
    off += 8
    attrs = {}
    if tag == 0:
        return attrs, off
    if tag != _NC_ATTRIBUTE:
        raise ValueError("not a classic netCDF attribute list")
    for _ in range(count):
        name, off = _read_name(buf, off)
        code, nelems = struct.unpack_from(">ii", buf, off)
        off += 8
        dt = np.dtype(_TYPES[code])
        nbytes = nelems * dt.itemsize
        raw = bytes(buf[off:off + nbytes])
        off += nbytes + (-nbytes % 4)
        attrs[name] = raw.decode() if code == 2 else np.frombuffer(raw, dtype=dt).copy()
    return attrs, off


def read_file(path: str) -> dict:
    """{'dims': {name: length}, 'attrs': {...}, 'vars': {name: (dims,
    ndarray)}} of a classic (CDF-1) file without record variables."""
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:4] != _MAGIC:
        raise ValueError(f"{path}: not a classic-format (CDF-1) netCDF file")
    off = 8
    tag, count = struct.unpack_from(">ii", buf, off)
    off += 8
    dims = []
    if tag == _NC_DIMENSION:
        for _ in range(count):
            name, off = _read_name(buf, off)
            (length,) = struct.unpack_from(">i", buf, off)
            off += 4
            if length == 0:
                raise ValueError(f"{path}: record dimensions are not supported")
            dims.append((name, length))
    attrs, off = _read_attrs(buf, off)
    tag, count = struct.unpack_from(">ii", buf, off)
    off += 8
    variables = {}
    for _ in range(count if tag == _NC_VARIABLE else 0):
        name, off = _read_name(buf, off)
        (nd,) = struct.unpack_from(">i", buf, off)
        off += 4
        ids = struct.unpack_from(">" + "i" * nd, buf, off)
        off += 4 * nd
        _, off = _read_attrs(buf, off)
        code, _vsize, begin = struct.unpack_from(">iii", buf, off)
        off += 12
        shape = tuple(dims[i][1] for i in ids)
        dt = np.dtype(_TYPES[code])
        n = int(np.prod(shape)) if shape else 1
        data = np.frombuffer(buf, dtype=dt, count=n, offset=begin).reshape(shape).copy()
        variables[name] = (tuple(dims[i][0] for i in ids), data)
    return {"dims": dict(dims), "attrs": attrs, "vars": variables}


def _run_attrs(p, with_basis: bool):
    a = []
    if with_basis:
        a.append(("N_basis", np.int32(p.n_basis)))
    a += [("N_1", np.int32(p.n_1)), ("N_2", np.int32(p.n_2)), ("N_3", np.int32(p.n_3)),
          ("Number of Species", np.int32(p.n_species)), ("Lattice Type", p.lattice.strip())]
    return a


def write_config(path: str, config, p) -> None:
    """ncdf_grid_state_writer.  config: the doubled grid C-ordered (z, y, x)
    (or (z, y, x, b)) of species codes; p: a RunParams-like object (n_basis,
    n_1..n_3, n_species, lattice, species_concentrations[0..n_species])."""
    c = np.asarray(config)
    if c.ndim == 3:
        c = c[..., None]
    nz, ny, nx, nb = c.shape
    attrs = _run_attrs(p, True) + [("Concentrations", np.asarray(p.species_concentrations, dtype=np.float64))]
    dims = [("b", nb), ("x", nx), ("y", ny), ("z", nz)]
    with open(path, "wb") as f:
        f.write(_encode(dims, attrs, [("configuration", ["z", "y", "x", "b"], c.astype(">i2"))]))


def read_config(path: str, p) -> np.ndarray:
    """ncdf_config_reader: the configuration as int8 C-ordered (z, y, x),
    after the reference's checks of lattice, N_basis and N_1..N_3 against p
    (ValueError with the reference's message where it stops)."""
    d = read_file(path)
    a = d["attrs"]
    for key in ("N_basis", "N_1", "N_2", "N_3", "Lattice Type"):
        if key not in a:
            raise ValueError(f"{path}: attribute {key!r} missing")
    checks = [(a["Lattice Type"].strip() != p.lattice.strip(), "Lattice types"),
              (int(a["N_basis"][0]) != p.n_basis, "n_basis values"),
              (int(a["N_1"][0]) != p.n_1, "n_1 values"), (int(a["N_2"][0]) != p.n_2, "n_2 values"),
              (int(a["N_3"][0]) != p.n_3, "n_3 values")]
    for bad, what in checks:
        if bad:
            raise ValueError(f"{what} do not match in ncdf_config_reader()")
    _, data = d["vars"]["configuration"]
    want = (2 * p.n_3, 2 * p.n_2, 2 * p.n_1, p.n_basis)
    if data.shape != want:
        raise ValueError(f"{path}: configuration has shape {data.shape}, expected {want}")
    out = data.astype(np.int8)
    return out[..., 0] if p.n_basis == 1 else out


def write_radial_density(path: str, rho, r, T, U, p) -> None:
    """ncdf_radial_density_writer.  rho: C-ordered (T, r, j, i) -- the
    Fortran rho(i, j, r, T); r, T, U: 1-D.  p additionally gives
    interaction_file and wc_range."""
    rho = np.asarray(rho, dtype=">f8")
    nT, nr, nj, ni = rho.shape
    r = np.asarray(r, dtype=">f8").ravel()
    T = np.asarray(T, dtype=">f8").ravel()
    U = np.asarray(U, dtype=">f8").ravel()
    attrs = _run_attrs(p, False) + [
        ("Interaction file", p.interaction_file.strip()),
        ("Concentrations", np.asarray(p.species_concentrations, dtype=np.float64)),
        ("Warren-Cowley Range", np.int32(p.wc_range))]
    dims = [("i", ni), ("j", nj), ("r", nr), ("T", nT), ("r_i", r.size), ("T_i", T.size),
            ("U_i", U.size)]
    variables = [("rho data", ["T", "r", "j", "i"], rho), ("r data", ["r_i"], r),
                 ("T data", ["T_i"], T), ("U data", ["U_i"], U)]
    with open(path, "wb") as f:
        f.write(_encode(dims, attrs, variables))


def read_radial_density(path: str, p, n_steps: int):
    """ncdf_radial_density_reader: (rho C-ordered (T, r, j, i), U), after
    the reference's checks of lattice, species and range against p."""
    d = read_file(path)
    dims = d["dims"]
    lattice = d["attrs"].get("Lattice Type", "")
    checks = [(lattice.strip() != p.lattice.strip(), "Lattice types"),
              (dims.get("i") != p.n_species, "n_species values"),
              (dims.get("j") != p.n_species, "n_species values"),
              (dims.get("r") != p.wc_range, "wc_range values"),
              (dims.get("T") != n_steps, "n_steps values")]
    for bad, what in checks:
        if bad:
            raise ValueError(f"{what} do not match in ncdf_radial_density_reader()")
    return d["vars"]["rho data"][1], d["vars"]["U data"][1]


def write_grid_1d(path: str, data) -> None:
    """ncdf_writer_1d: "grid data" over dimension x (the Wang-Landau ln g)."""
    a = np.asarray(data, dtype=">f8").ravel()
    with open(path, "wb") as f:
        f.write(_encode([("x", a.size)], [], [("grid data", ["x"], a)]))


def write_order(path: str, order_of_T, temperature, p) -> None:
    """ncdf_order_writer.  order_of_T: C-ordered (T, 2n3, 2n2, 2n1, n_basis,
    n_species) -- the Fortran order(species, basis, x, y, z, T) -- as the
    annealing driver returns it.  The reference labels the six dimensions
    b, x, y, z, s, t in Fortran order whatever they hold (so "b" has
    n_species entries), and writes N_Basis (capital B) among the run's
    attributes."""
    o = np.asarray(order_of_T, dtype=">f8")
    nT, n3, n2, n1, nb, ns = o.shape
    T = np.asarray(temperature, dtype=">f8").ravel()
    attrs = [("N_Basis", np.int32(p.n_basis))] + _run_attrs(p, False) + [
        ("Interaction file", p.interaction_file.strip()),
        ("Concentrations", np.asarray(p.species_concentrations, dtype=np.float64)),
        ("Warren-Cowley Range", np.int32(p.wc_range))]
    dims = [("b", ns), ("x", nb), ("y", n1), ("z", n2), ("s", n3), ("t", nT), ("temp", T.size)]
    variables = [("grid data", ["t", "s", "z", "y", "x", "b"], o), ("temperature data", ["temp"], T)]
    with open(path, "wb") as f:
        f.write(_encode(dims, attrs, variables))
