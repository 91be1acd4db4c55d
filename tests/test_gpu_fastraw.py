"""FastRaw straight to and from device memory: the file streamed through
the pinned staging buffers into a device-resident ndarray (and a file of
several staging chunks), device-resident data written out, and a view
written through a contiguous device copy."""
import numpy as np
import pytest

import pdl_gb300 as P

pytestmark = pytest.mark.gpu


def test_device_round_trip(gpu, tmp_path):
    a = np.random.default_rng(1).standard_normal((300, 257)).astype(np.float32)
    x = P.pdl(a).to_device()
    name = str(tmp_path / "dev")
    P.writefraw(x, name)
    assert (tmp_path / "dev.hdr").read_text() == "9\n2\n257 300\n"
    y = P.readfraw(name, device=True)
    assert y.on_device and y.type == "float" and y.dims == (257, 300)
    assert np.array_equal(y.numpy(), a)
    # a reduction runs on the device-resident result directly
    assert np.allclose(P.sumover(y).numpy(), a.astype(np.float64).sum(-1), rtol=1e-5, atol=1e-4)


def test_device_read_of_several_chunks(gpu, tmp_path):
    # 80 MiB: three 32 MiB staging chunks, the last one partial
    n = 80 * (1 << 20) // 8
    a = np.arange(n, dtype=np.int64)
    name = str(tmp_path / "big")
    a.tofile(name)
    (tmp_path / "big.hdr").write_text(f"8\n1\n{n}\n")
    y = P.readfraw(name, device=True)
    got = y.numpy()
    assert got.dtype == np.int64 and np.array_equal(got, a)


def test_device_short_file_is_zero_filled(gpu, tmp_path):
    name = str(tmp_path / "short")
    np.array([1.5, 2.5], np.float64).tofile(name)
    (tmp_path / "short.hdr").write_text("10\n1\n5\n")
    assert P.readfraw(name, device=True).numpy().tolist() == [1.5, 2.5, 0.0, 0.0, 0.0]


def test_view_written_contiguously(gpu, tmp_path):
    a = np.arange(120, dtype=np.int32).reshape(4, 5, 6)
    v = P.pdl(a).xchg(0, 2)
    name = str(tmp_path / "view")
    P.writefraw(v, name)
    y = P.readfraw(name)
    assert y.dims == v.dims and np.array_equal(y.numpy(), v.numpy())


@pytest.mark.parametrize("name", ["seq_double", "seq_long", "seq_byte", "float_bad", "own_header"])
def test_device_read_of_files_pdl_wrote(gpu, name):
    """Files written by the reference PDL's writefraw, read into device memory."""
    from test_fastraw import GOLDEN, pdl_written
    t, dims, want, hdr = pdl_written()[name]
    y = P.readfraw(str(GOLDEN / name), header=str(GOLDEN / hdr) if hdr else None, device=True)
    assert y.on_device and y.type == t and y.dims == dims
    assert y.numpy().tobytes() == want.tobytes()


def test_mapfraw_device_results_reach_the_file(gpu, tmp_path):
    """An op's output on the device, brought back to the host, is in the file."""
    from test_fastraw import GOLDEN
    src = P.mapfraw(str(GOLDEN / "seq_double"), ReadOnly=True).to_device()
    name = str(tmp_path / "sums")
    out = P.mapfraw(name, Dims=[4, 3], Creat=True)
    P.sumover(src, out=out)
    out.to_host()
    want = (np.arange(60, dtype=np.float64).reshape(3, 4, 5) * 1.5 - 7).sum(-1)
    assert np.fromfile(name, dtype=np.float64).tobytes() == want.tobytes()
    assert P.readfraw(name).numpy().tobytes() == want.tobytes()


def test_device_read_from_a_pipe_streams_through_staging(gpu, tmp_path):
    """A FastRaw 'file' that cannot be mapped (a named pipe) goes through the
    pinned staging buffers: several 32 MiB chunks and a short tail."""
    import os
    import threading
    n = (80 << 20) // 8 + 123                       # 2.5 staging chunks of float64
    a = np.arange(n, dtype=np.float64) * 0.5 - 7
    name = str(tmp_path / "pipe")
    os.mkfifo(name)
    with open(name + ".hdr", "w") as f:
        f.write(f"10\n1\n{n + 1000}\n")               # 1000 more than the pipe holds
    w = threading.Thread(target=lambda: open(name, "wb").write(a.tobytes()), daemon=True)
    w.start()
    y = P.readfraw(name, device=True)
    w.join(timeout=60)
    got = y.numpy()
    assert got[:n].tobytes() == a.tobytes() and np.all(got[n:] == 0)
