"""Seeded synthetic microstructures and the reference's voxel file formats.

The reference reads its geometry from text ``.geom`` or binary ``.fgeo``
files (src/io/VoxelIO.cpp:89-159) and publishes no data set, so every
workload here is generated from a seed:

* ``spheres``: overlapping solid spheres with uniform random centres in a
  periodic cube (minimum-image distance, voxel centres at i + 1/2), added one
  at a time until the porosity drops to the target.
* ``gaussian_field``: white N(0, 1) noise convolved periodically with a
  Gaussian of correlation length ``corr_len`` (a spectral multiply by
  exp(-2 pi^2 l^2 |xi|^2)), thresholded at its porosity quantile so that the
  fluid fraction equals the target; isolated fluid clusters are kept.

Masks are uint8 arrays of shape (nz, ny, nx), x fastest, 1 = fluid and
0 = solid, the reference's BinaryMedium convention
(src/geometry/BinaryMedium.cpp:9-11).
"""
from __future__ import annotations

import re
import struct

import numpy as np

FLUID_ID = 1
SOLID_ID = 2


def spheres(n, radius: float, porosity: float, seed: int, radius_max: float | None = None):
    """Union of random spheres in an n^3 (or (nz, ny, nx)) periodic cell.

    With ``radius_max`` each sphere draws its radius uniformly from
    [radius, radius_max].
    """
    shape = (n, n, n) if np.isscalar(n) else tuple(n)
    nz, ny, nx = shape
    rng = np.random.default_rng(seed)
    solid = np.zeros(shape, dtype=bool)
    total = solid.size
    n_solid = 0
    target_solid = (1.0 - porosity) * total
    while n_solid < target_solid:
        c = rng.uniform(0.0, 1.0, size=3) * np.array([nx, ny, nz])
        r = radius if radius_max is None else rng.uniform(radius, radius_max)
        rc = int(np.ceil(r)) + 1
        ix = np.arange(int(np.floor(c[0])) - rc, int(np.floor(c[0])) + rc + 1)
        iy = np.arange(int(np.floor(c[1])) - rc, int(np.floor(c[1])) + rc + 1)
        iz = np.arange(int(np.floor(c[2])) - rc, int(np.floor(c[2])) + rc + 1)
        dx = ix + 0.5 - c[0]
        dy = iy + 0.5 - c[1]
        dz = iz + 0.5 - c[2]
        d2 = dz[:, None, None] ** 2 + dy[None, :, None] ** 2 + dx[None, None, :] ** 2
        inside = d2 <= r * r
        zz = np.mod(iz, nz)[:, None, None]
        yy = np.mod(iy, ny)[None, :, None]
        xx = np.mod(ix, nx)[None, None, :]
        zz, yy, xx = np.broadcast_arrays(zz, yy, xx)
        sel = (zz[inside], yy[inside], xx[inside])
        before = solid[sel]
        solid[sel] = True
        n_solid += int(np.count_nonzero(~before))
    return (~solid).astype(np.uint8)


def gaussian_field(n, corr_len: float, porosity: float, seed: int):
    """Thresholded Gaussian random field; fluid = field below its porosity quantile."""
    shape = (n, n, n) if np.isscalar(n) else tuple(n)
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(shape)
    spec = np.fft.rfftn(noise)
    kz = np.fft.fftfreq(shape[0])[:, None, None]
    ky = np.fft.fftfreq(shape[1])[None, :, None]
    kx = np.fft.rfftfreq(shape[2])[None, None, :]
    filt = np.exp(-2.0 * np.pi ** 2 * corr_len ** 2 * (kx ** 2 + ky ** 2 + kz ** 2))
    field = np.fft.irfftn(spec * filt, s=shape, axes=(0, 1, 2))
    flat = field.ravel()
    k = int(round(porosity * flat.size))
    fluid = np.zeros(flat.size, dtype=np.uint8)
    if k > 0:
        order = np.argsort(flat, kind="stable")
        fluid[order[:k]] = 1
    return fluid.reshape(shape)


BATCH_EDGES = (48, 64, 80, 96, 128, 160)


def batch_cell(seed: int) -> np.ndarray:
    """One cell of the uneven-size batch workload: the edge is drawn uniformly
    from BATCH_EDGES and the porosity uniformly from [0.3, 0.8] with
    default_rng(seed); even seeds are overlapping spheres with radii uniform
    in [3, 10], odd seeds Gaussian random fields of correlation length 6."""
    rng = np.random.default_rng(seed)
    edge = int(rng.choice(list(BATCH_EDGES)))
    phi = float(rng.uniform(0.3, 0.8))
    if seed % 2 == 0:
        return spheres(edge, 3.0, phi, seed=seed, radius_max=10.0)
    return gaussian_field(edge, 6.0, phi, seed=seed)


def porosity(mask: np.ndarray) -> float:
    return float(np.count_nonzero(mask)) / mask.size


def to_ids(mask: np.ndarray) -> np.ndarray:
    """Material ids for a fluid mask (fluid 1, solid 2)."""
    return np.where(mask != 0, FLUID_ID, SOLID_ID).astype(np.uint32)


def write_fgeo(path: str, mask_or_ids: np.ndarray, ids: bool = False) -> None:
    """Write the reference's binary .fgeo format (src/io/VoxelIO.cpp:99-107):
    magic FGEO, version 1, value_type 2 (uint16), 2 reserved bytes, nx, ny, nz
    as little-endian uint64, then one uint16 per voxel, x fastest."""
    vals = mask_or_ids if ids else to_ids(mask_or_ids)
    nz, ny, nx = vals.shape
    with open(path, "wb") as f:
        f.write(b"FGEO" + bytes([1, 2, 0, 0]))
        f.write(struct.pack("<QQQ", nx, ny, nz))
        f.write(np.ascontiguousarray(vals, dtype="<u2").tobytes())


def read_fgeo(path: str) -> np.ndarray:
    """Read a .fgeo file; returns uint32 material ids of shape (nz, ny, nx)."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < 32 or data[:4] != b"FGEO":
        raise ValueError("invalid .fgeo magic: " + path)
    if data[4] != 1:
        raise ValueError("unsupported .fgeo version %d" % data[4])
    vt = data[5]
    if vt not in (1, 2):
        raise ValueError("unsupported .fgeo value_type %d" % vt)
    nx, ny, nz = struct.unpack("<QQQ", data[8:32])
    dt = "<u4" if vt == 1 else "<u2"
    count = nx * ny * nz
    if len(data) != 32 + count * np.dtype(dt).itemsize:
        raise ValueError(".fgeo payload size mismatch: " + path)
    return np.frombuffer(data, dtype=dt, offset=32).astype(np.uint32).reshape(nz, ny, nx)


_LEADING_INT = re.compile(r"\s*([+-]?\d+)")


def strip_comment(line: str) -> str:
    """The part of a line before its first "#" or ";" (the reference's comment rule)."""
    cut = min((i for i in (line.find("#"), line.find(";")) if i >= 0), default=-1)
    return line if cut < 0 else line[:cut]


def _line_ints(line: str):
    """The integers a C++ ``istringstream >> int`` loop reads from a line:
    leading integer tokens, up to the first token that is not one."""
    pos = 0
    while True:
        m = _LEADING_INT.match(line, pos)
        if not m:
            return
        yield int(m.group(1))
        pos = m.end()


def read_geom_text(path: str) -> np.ndarray:
    """Read the reference's text geometry (src/io/VoxelIO.cpp:47-86): '#' and
    ';' start comments, the first non-empty line gives nx ny nz, then one
    integer material id per voxel (x fastest) in any line layout; values past
    nx*ny*nz are ignored.  Returns int64 material ids of shape (nz, ny, nx)."""
    with open(path) as f:
        lines = iter(f.read().splitlines())
    dims = None
    for line in lines:
        body = strip_comment(line)
        if not body.strip():
            continue
        dims = list(_line_ints(body))[:3]
        break
    if dims is None or len(dims) < 3 or min(dims) < 0:
        raise ValueError("VoxelIO::load_text expected first non-comment line: nx ny nz")
    nx, ny, nz = dims
    count = nx * ny * nz
    vals = []
    for line in lines:
        if len(vals) >= count:
            break
        for v in _line_ints(strip_comment(line)):
            vals.append(v)
            if len(vals) == count:
                break
    if len(vals) < count:
        raise ValueError("VoxelIO::load_text insufficient voxel values")
    return np.asarray(vals, dtype=np.int64).reshape(nz, ny, nx)


def load_ids(path: str) -> np.ndarray:
    """Material ids from a geometry file, by extension as the reference's
    VoxelIO::load does (src/io/VoxelIO.cpp:159-164): ``.fgeo`` is binary,
    anything else text."""
    return read_fgeo(path) if path.endswith(".fgeo") else read_geom_text(path)


def load_mask(path: str, fluid_id: int = FLUID_ID) -> np.ndarray:
    """VoxelIO::load: the fluid mask (1 where the id equals ``fluid_id``)."""
    return (load_ids(path) == fluid_id).astype(np.uint8)
