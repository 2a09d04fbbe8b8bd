"""GPU: file and stream I/O from ranks over the device -> host request channel.

The `file_io` device program (csrc/programs/prog_tests.cu) exercises MPI-IO (open modes and their
errors, explicit offsets, individual and shared file pointers, a contiguous and a non-contiguous file
view, size, delete-on-close) and the gpumpi stdio functions; this test checks the files it leaves, byte
for byte, and the line gpumpi_printf wrote to the process's standard output.  The reference's own I/O
tests (tests/test_io_file_open.cu, test_io_file_access.cu, test_io_file_write.cu) cover the open modes,
read-back, size and views; there, read and write calls return element counts, here they return
MPI_SUCCESS and report the amount in the status, as the MPI standard specifies."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

K, NW = 300, 50


@pytest.mark.parametrize("n", [1, 8, 33])
def test_mpi_io_and_stdio(gpulib, tmp_path, capfd, n):
    d = str(tmp_path).encode() + b"\0"
    dirt = torch.tensor(list(d), dtype=torch.uint8, device="cuda")
    ok = torch.zeros(n, dtype=torch.uint8, device="cuda")
    oi = torch.zeros((n, 64), dtype=torch.int64, device="cuda")
    od = torch.zeros((n, 64), dtype=torch.float64, device="cuda")
    with gpulib.World(n, timeout_s=20.0) as w:
        rc = w.run_program(gpulib.TESTS["file_io"], p=(ok, oi, od, dirt))
    torch.cuda.synchronize()
    oi_h = oi.cpu().numpy()
    assert rc == 0 and bool(ok.all()), ("first failed check per rank", oi_h[:, 0], oi_h[:, 1:7])

    blk = np.fromfile(tmp_path / "io_block.bin", dtype=np.int32)
    assert np.array_equal(blk, (np.arange(n)[:, None] * 1000 + np.arange(K)[None, :]).ravel())

    view = np.fromfile(tmp_path / "io_view.bin", dtype=np.int32).reshape(2, n, NW)
    want = np.arange(n)[None, :, None] * 100 + (np.arange(2)[:, None, None] * NW + np.arange(NW)[None, None, :])
    assert np.array_equal(view, want)

    shared = np.fromfile(tmp_path / "io_shared.bin", dtype=np.int32)
    assert sorted(shared.tolist()) == list(range(n))

    assert not (tmp_path / "io_tmp.bin").exists()   # MPI_MODE_DELETE_ON_CLOSE

    text = (tmp_path / "io_stdio.txt").read_text()
    line = "rank %d of %d pi %.6f name %s hex %#x pad [%5d] [%-4s] %c%%\n" % (0, n, 3.14159265358979, "gb300", 255,
                                                                           42, "ab", "z")
    assert text == line + "second line\n"
    out = capfd.readouterr().out
    assert ("gpumpi_printf from rank %d of %d: %s %.3e\n" % (0, n, "ok", 1234.5)) in out


def test_channel_survives_many_requests(gpulib, tmp_path):
    """Ranks keep the channel busy back to back (more requests than ring slots, every rank at once)."""
    n = 64
    d = str(tmp_path).encode() + b"\0"
    dirt = torch.tensor(list(d), dtype=torch.uint8, device="cuda")
    with gpulib.World(n, timeout_s=20.0) as w:
        for _ in range(3):
            ok = torch.zeros(n, dtype=torch.uint8, device="cuda")
            oi = torch.zeros((n, 64), dtype=torch.int64, device="cuda")
            od = torch.zeros((n, 64), dtype=torch.float64, device="cuda")
            rc = w.run_program(gpulib.TESTS["file_io"], p=(ok, oi, od, dirt))
            assert rc == 0 and bool(ok.all()), oi.cpu().numpy()[:, 0]
