"""Fortran sequential-unformatted record files (the reference's .dat contract).

Every model, CPML, initial-condition and source file the reference reads is
one record written by gfortran (src/fortran/seidartio.f08:161-292): a 4-byte
little-endian length, the payload (column-major array), the same length
again.  Payloads over 2**31 - 9 bytes are split into subrecords whose head
marker is negative when another subrecord follows.
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

_MAX = 2147483639


def write_record(path, array) -> None:
    """Write ``array`` (any dtype, written in Fortran order) as one record."""
    data = np.asfortranarray(array).tobytes(order="F")
    with open(path, "wb") as f:
        off, first = 0, True
        while True:
            n = min(_MAX, len(data) - off)
            more = off + n < len(data)
            f.write(struct.pack("<i", -n if more else n))
            f.write(data[off:off + n])
            f.write(struct.pack("<i", n if first else -n))
            off += n
            first = False
            if not more:
                break


def read_record(path, dtype=np.float64, shape=None) -> np.ndarray:
    """Read one record; reshape in Fortran order when ``shape`` is given."""
    raw = bytearray()
    with open(path, "rb") as f:
        while True:
            head = f.read(4)
            if len(head) != 4:
                raise ValueError(f"{path}: truncated record marker")
            (h,) = struct.unpack("<i", head)
            n = -h if h < 0 else h
            chunk = f.read(n)
            if len(chunk) != n:
                raise ValueError(f"{path}: truncated record")
            raw += chunk
            if len(f.read(4)) != 4:
                raise ValueError(f"{path}: missing trailing marker")
            if h >= 0:
                break
    a = np.frombuffer(bytes(raw), dtype=dtype)
    if shape is not None:
        a = a.reshape(shape, order="F")
    return a


def _zstd_lib():
    import ctypes
    import ctypes.util
    for name in ("libzstd.so.1", ctypes.util.find_library("zstd")):
        if not name:
            continue
        try:
            L = ctypes.CDLL(name)
        except OSError:
            continue
        L.ZSTD_getFrameContentSize.restype = ctypes.c_ulonglong
        L.ZSTD_getFrameContentSize.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
        L.ZSTD_decompress.restype = ctypes.c_size_t
        L.ZSTD_decompress.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t]
        L.ZSTD_isError.restype = ctypes.c_uint
        L.ZSTD_isError.argtypes = [ctypes.c_size_t]
        return L
    return None


def _raw_frame(buf: bytes) -> bytes:
    """Content of a zstd frame made of raw blocks only (RFC 8878: magic,
    frame header, 3-byte block headers); other block types need libzstd."""
    if buf[:4] != b"\x28\xb5\x2f\xfd":
        raise ValueError("not a zstd frame")
    fhd = buf[4]
    single = (fhd >> 5) & 1
    fcs_size = {0: 1 if single else 0, 1: 2, 2: 4, 3: 8}[fhd >> 6]
    did_size = {0: 0, 1: 1, 2: 2, 3: 4}[fhd & 3]
    pos = 5 + (0 if single else 1) + did_size + fcs_size
    out = bytearray()
    while True:
        hdr = buf[pos] | (buf[pos + 1] << 8) | (buf[pos + 2] << 16)
        pos += 3
        last, btype, size = hdr & 1, (hdr >> 1) & 3, hdr >> 3
        if btype != 0:
            raise ValueError("compressed zstd block: libzstd is needed to read it")
        out += buf[pos:pos + size]
        pos += size
        if last:
            return bytes(out)


def read_zstd(path) -> bytes:
    """Decompressed content of a one-frame .zst file (libzstd when it loads,
    else frames of raw blocks)."""
    import ctypes
    buf = Path(path).read_bytes()
    L = _zstd_lib()
    if L is None:
        return _raw_frame(buf)
    n = L.ZSTD_getFrameContentSize(buf, len(buf))
    if n >= (1 << 64) - 2:
        raise ValueError(f"{path}: zstd frame without a content size")
    out = ctypes.create_string_buffer(max(int(n), 1))
    got = L.ZSTD_decompress(out, int(n), buf, len(buf))
    if L.ZSTD_isError(got):
        raise ValueError(f"{path}: zstd decompression failed")
    return out.raw[:got]


def block_name(prefix: str, first: int, last: int, xind: int, yind: int, zind: int) -> str:
    """2.5D zstd block file name (src/fortran/cpmlfdtd.f08:1300-1302, :3318-3320)."""
    return f"{prefix}.{first:06d}-{last:06d}.{xind}.{yind}.{zind}.blk.zst"


def read_block(path, onx: int, onz: int) -> np.ndarray:
    """One 2.5D output block as float32 (onx, 1, onz, 3, steps), Fortran order
    (seidartio.f08:604-677)."""
    a = np.frombuffer(read_zstd(path), dtype=np.float32)
    steps = a.size // (onx * onz * 3)
    return a.reshape((onx, 1, onz, 3, steps), order="F")


def snapshot_name(channel: str, it: int, xind: int, zind: int, yind: int | None = None) -> str:
    """write_image2 / write_image3 file names (src/fortran/seidartio.f08:380, :414)."""
    if yind is None:
        return f"{channel}.{it:06d}.{xind}.{zind}.dat"
    return f"{channel}.{it:06d}.{xind}.{yind}.{zind}.dat"


def write_problem(problem, directory, source_type: str = "ac", json_extra: dict | None = None) -> Path:
    """Write a Problem as the reference's input files plus input.json (the
    frontend's role): material, CPML, initial-condition and source records."""
    import json

    from .api import FIELD_SLOTS, MODEL_SLOTS, SRC_SLOTS
    from ._lib import ELECTROMAG2, ELECTROMAG3, ELECTROMAG25, SEISMIC25

    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    fam = problem.family
    seismic = fam not in (ELECTROMAG2, ELECTROMAG25, ELECTROMAG3)
    for name in MODEL_SLOTS[fam]:
        fname = {"kappa": "kappa_cpml", "kappa_half": "kappa_half_cpml", "acoef": "acoef_cpml",
                 "acoef_half": "acoef_half_cpml", "bcoef": "bcoef_cpml", "bcoef_half": "bcoef_half_cpml"}.get(name, name)
        write_record(d / f"{fname}.dat", np.asarray(problem.model[name], dtype=np.float64))
    # alpha grids are read by the reference but unused in its loops
    write_record(d / "alpha_cpml.dat", np.zeros(problem.shape))
    write_record(d / "alpha_half_cpml.dat", np.zeros(problem.shape))
    prefix = "seismicsource" if seismic else "electromagneticsource"
    for name in SRC_SLOTS[fam]:
        s = problem.src.get(name)
        write_record(d / f"{prefix}{name}.dat", np.zeros(problem.time_steps) if s is None else np.asarray(s, np.float64))
    dt = np.complex128 if problem.is_complex else np.float64
    for name in FIELD_SLOTS[fam][:(2 if fam in (ELECTROMAG2,) or fam == 1 else 3)]:
        f = problem.fields0.get(name)
        key = "initialcondition" + (name[0].upper() + name[1:])
        write_record(d / f"{key}.dat", np.zeros(problem.shape, dtype=dt) if f is None else np.asarray(f, dt))
    dim = 3 if problem.is3d else (2.5 if fam in (SEISMIC25, ELECTROMAG25) else 2)
    src = {"x": 0.0, "y": 0.0, "z": 0.0, "xind": problem.xind, "yind": problem.yind, "zind": problem.zind,
           "source_frequency": problem.meta.get("f0", 0.0), "x-z_rotation": 0.0, "x-y_rotation": 0.0,
           "y-z_rotation": 0.0, "amplitude": 1.0, "source_type": source_type, "source_wavelet": "ricker",
           "dt": problem.dt, "time_steps": problem.time_steps}
    pw = problem.plane_wave
    if pw:
        src.update({"source_type": pw.get("kind", "pw"), "source_wavelet": pw.get("wavelet", "gaus0"),
                    "source_frequency": pw["frequency"], "amplitude": pw.get("amplitude", 1.0),
                    "x-z_rotation": pw.get("x_z_rotation", 0.0), "x-y_rotation": pw.get("x_y_rotation", 0.0),
                    "y-z_rotation": pw.get("y_z_rotation", 0.0)})
    js = {"Domain": {"dim": dim, "nx": problem.nx - 2 * problem.cpml,
                     "ny": (problem.ny - 2 * problem.cpml) if problem.is3d else 1,
                     "nz": problem.nz - 2 * problem.cpml, "dx": problem.dx, "dy": problem.dy, "dz": problem.dz,
                     "cpml": problem.cpml, "nmats": 1, "image_file": "model.png"},
          "Seismic": {"Source": src}, "Electromagnetic": {"Source": src}}
    if json_extra:
        js.update(json_extra)
    (d / "input.json").write_text(json.dumps(js, indent=2))
    return d / "input.json"
