"""The raw dose file reader on a file written here (no GPU)."""
import numpy as np
import pytest


def test_read_raw(dpm, tmp_path):
    nx, ny, nz = 3, 4, 5
    dose = np.arange(nx * ny * nz, dtype="<f8") * 1e-15
    rel = np.linspace(0, 1, nx * ny * nz).astype("<f8")
    with open(tmp_path / "x.raw", "wb") as f:
        f.write(b"DPMXDOSE")
        f.write(np.array([1, nx, ny, nz], dtype="<i4").tobytes())
        f.write(np.array([1.0, 2.0, 3.0, -1.5, -4.0, 0.0], dtype="<f8").tobytes())
        f.write(np.array([1000, 10], dtype="<i8").tobytes())
        f.write(dose.tobytes())
        f.write(rel.tobytes())
    d, r, head = dpm.read_dose_raw(tmp_path / "x.raw")
    assert d.shape == (nz, ny, nx)
    np.testing.assert_array_equal(d.reshape(-1), dose)
    np.testing.assert_array_equal(r.reshape(-1), rel)
    assert head["histories"] == 1000 and head["batches"] == 10 and head["voxel_mm"] == (1.0, 2.0, 3.0)


def test_read_raw_rejects_other_files(dpm, tmp_path):
    (tmp_path / "y.raw").write_bytes(b"NOTADOSEFILE" + bytes(64))
    with pytest.raises(dpm.DpmxError):
        dpm.read_dose_raw(tmp_path / "y.raw")
