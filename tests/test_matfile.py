"""PSF files in MATLAB v7.3 (HDF5) format: sid_gb300.matfile reads them
without an HDF5 library (sid_main.m:30 psf_ballistic = matfile(psffile);
save_psf_fast.m:59-70 writes H, Nnum, CAindex with h5create / h5write)."""
import os

import numpy as np
import pytest

from sid_gb300 import matfile
from tests.h5_writer import write_mat73


def test_reads_a_matlab_written_hdf5_file():
    """A file MATLAB itself wrote with save -v7.3 (the HDF5 MAT-file that
    SciPy's test data carries; its variable is pi/4 * (0:8))."""
    scipy = pytest.importorskip("scipy")
    path = os.path.join(os.path.dirname(scipy.__file__), "io", "matlab", "tests", "data", "testhdf5_7.4_GLNX86.mat")
    if not os.path.exists(path):
        pytest.skip("SciPy's HDF5 MAT-file test data is not installed")
    v = matfile.matfile_read(path)
    assert list(v) == ["testdouble"]
    np.testing.assert_array_equal(v["testdouble"], (np.pi / 4 * np.arange(9))[None, :])


@pytest.mark.parametrize("chunked", [False, True])
def test_psf_round_trip(tmp_path, chunked):
    rng = np.random.default_rng(0)
    M, N, Z = 9, 3, 4
    H = np.asfortranarray(rng.random((M, M, N, N, Z), dtype=np.float32))
    CA = np.asfortranarray(np.stack([np.arange(1, Z + 1), M + 1 - np.arange(1, Z + 1)], 1).astype(np.float64))
    path = str(tmp_path / "psf.mat")
    write_mat73(path, {"H": H, "Nnum": np.float64(N), "CAindex": CA},
                chunks={"H": (M, M, N, N, 2)} if chunked else None)
    psf = matfile.load_psf(path)
    assert psf["Nnum"] == N
    assert psf["H"].shape == H.shape and psf["H"].flags.f_contiguous
    np.testing.assert_array_equal(psf["H"], H)
    np.testing.assert_array_equal(psf["CAindex"], CA)


def test_rejects_non_hdf5(tmp_path):
    p = tmp_path / "x.mat"
    p.write_bytes(b"MATLAB 5.0 MAT-file" + b"\x00" * 2000)
    with pytest.raises(matfile.MatFileError):
        matfile.matfile_read(str(p))
