"""Fortran sequential-unformatted records (the .dat file contract), host only."""
import struct

import numpy as np

from seidart_gpu import fortran_io as fio


def test_record_round_trip(tmp_path):
    a = np.asfortranarray(np.arange(12.0).reshape(3, 4))
    p = tmp_path / "a.dat"
    fio.write_record(p, a)
    raw = p.read_bytes()
    assert struct.unpack("<i", raw[:4])[0] == a.nbytes
    assert struct.unpack("<i", raw[-4:])[0] == a.nbytes
    # column-major payload, like write(unit) image_data in gfortran
    assert np.array_equal(np.frombuffer(raw[4:-4], dtype=np.float64), a.ravel(order="F"))
    b = fio.read_record(p, np.float64, (3, 4))
    assert np.array_equal(a, b)


def test_complex_and_float32_records(tmp_path):
    c = np.asfortranarray((np.arange(6) + 1j * np.arange(6)).reshape(2, 3))
    fio.write_record(tmp_path / "c.dat", c)
    assert np.array_equal(fio.read_record(tmp_path / "c.dat", np.complex128, (2, 3)), c)
    f = np.float32(np.linspace(0, 1, 7))
    fio.write_record(tmp_path / "f.dat", f)
    assert np.array_equal(fio.read_record(tmp_path / "f.dat", np.float32), f)


def test_subrecord_reading(tmp_path):
    """Payloads split into subrecords (negative head markers) are joined."""
    p = tmp_path / "s.dat"
    a = np.arange(10.0)
    d = a.tobytes()
    with open(p, "wb") as f:
        f.write(struct.pack("<i", -40)); f.write(d[:40]); f.write(struct.pack("<i", 40))
        f.write(struct.pack("<i", 40)); f.write(d[40:]); f.write(struct.pack("<i", -40))
    assert np.array_equal(fio.read_record(p), a)


def test_snapshot_names():
    assert fio.snapshot_name("Vx", 7, 128, 40) == "Vx.000007.128.40.dat"
    assert fio.snapshot_name("Vz", 123456, 1, 2, yind=3) == "Vz.123456.1.3.2.dat"
