"""PDL::IO::FastRaw through the C ABI on host memory (no GPU): the cases of
the reference's t/fastraw.t (write then read back, gluefraw, a custom
header), the header text exactly as _writefrawhdr writes it, a short file
read as zeroes, and the header errors.  Device-resident reads and writes,
and views (written through a device copy), are in test_gpu_fastraw.py."""
import numpy as np
import pytest

import pdl_gb300 as P


def startdata():
    return P.pdl(np.array([[2.0, 3], [4, 5], [6, 7]]))    # PDL dims (2, 3)


def test_write_read_round_trip(tmp_path):
    name = str(tmp_path / "tmp0")
    x = startdata()
    P.writefraw(x, name)
    assert (tmp_path / "tmp0").is_file() and (tmp_path / "tmp0.hdr").is_file()
    # type id (double = 10 in PDL's order), ndims, dims
    assert (tmp_path / "tmp0.hdr").read_text() == "10\n2\n2 3\n"
    y = P.readfraw(name)
    assert y.type == "double" and y.dims == (2, 3)
    assert np.array_equal(y.numpy(), x.numpy())


def test_gluefraw(tmp_path):
    name = str(tmp_path / "tmp0.g")
    P.writefraw(startdata(), name)
    P.gluefraw(P.pdl(np.array([10.0, 11])), name)
    y = P.readfraw(name)
    assert np.array_equal(y.numpy(), np.array([[2.0, 3], [4, 5], [6, 7], [10, 11]]))
    with pytest.raises(P.PDLError, match="has type 'long' but file has type"):
        P.gluefraw(P.pdl(np.array([1, 2], np.int32)), name)
    with pytest.raises(P.PDLError, match="incompatible lower dims"):
        P.gluefraw(P.pdl(np.array([1.0, 2, 3])), name)


def test_custom_header(tmp_path):
    name, header = str(tmp_path / "tmp0"), str(tmp_path / "headerfile")
    x = startdata()
    P.writefraw(x, name, header=header)
    assert (tmp_path / "headerfile").is_file() and not (tmp_path / "tmp0.hdr").exists()
    assert np.array_equal(P.readfraw(name, header=header).numpy(), x.numpy())


NP = {"byte": np.uint8, "short": np.int16, "long": np.int32, "longlong": np.int64,
      "float": np.float32, "double": np.float64}


@pytest.mark.parametrize("t", list(NP))
def test_types(tmp_path, t):
    a = np.random.default_rng(0).integers(0, 100, size=(4, 5, 6)).astype(NP[t])
    x = P.pdl(a)
    name = str(tmp_path / f"f_{t}")
    P.writefraw(x, name)
    y = P.readfraw(name)
    assert y.type == t and y.dims == (6, 5, 4)
    assert np.array_equal(y.numpy(), a)


def test_short_file_reads_zeroes_and_header_errors(tmp_path):
    name = str(tmp_path / "short")
    (tmp_path / "short").write_bytes(np.array([1.5, 2.5], np.float64).tobytes())
    (tmp_path / "short.hdr").write_text("10\n1\n4\n")
    assert P.readfraw(name).numpy().tolist() == [1.5, 2.5, 0.0, 0.0]
    (tmp_path / "bad.hdr").write_text("10\n2\n4\n")
    (tmp_path / "bad").write_bytes(b"")
    with pytest.raises(P.PDLError, match="Format error reading fraw header file"):
        P.readfraw(str(tmp_path / "bad"))
    (tmp_path / "trunc.hdr").write_text("10\n1\n")
    (tmp_path / "trunc").write_bytes(b"")
    with pytest.raises(P.PDLError, match="Format error in"):
        P.readfraw(str(tmp_path / "trunc"))
    with pytest.raises(P.PDLError, match="Couldn't open"):
        P.readfraw(str(tmp_path / "missing"))


def test_zero_dims_header_and_glue_errors(tmp_path):
    # a 0-dim ndarray: "10\n0\n\n" (_writefrawhdr joins no dims)
    name = str(tmp_path / "scalar")
    P.writefraw(P.pdl(np.array(2.5)), name)
    assert (tmp_path / "scalar.hdr").read_text() == "10\n0\n\n"
    y = P.readfraw(name)
    assert y.dims == () and float(y.numpy()) == 2.5
    # gluefraw wants a file of at least 2 dims (FastRaw.pm:336)
    one = str(tmp_path / "one")
    P.writefraw(P.pdl(np.array([1.0, 2.0])), one)
    with pytest.raises(P.PDLError, match="needs at least 2 dims"):
        P.gluefraw(P.pdl(np.array([3.0, 4.0])), one)
    with pytest.raises(P.PDLError, match="must be real filename"):
        P.gluefraw(P.pdl(np.array([3.0])), str(tmp_path / "nofile"))


def test_header_type_outside_this_path(tmp_path):
    (tmp_path / "ld").write_bytes(b"")
    (tmp_path / "ld.hdr").write_text("11\n1\n2\n")        # long double
    with pytest.raises(P.PDLError, match="not on this path"):
        P.readfraw(str(tmp_path / "ld"))


def test_gluefraw_lower_dims_compare_like_the_reference(tmp_path):
    """FastRaw.pm:338-339 compares $pdl->shape with pdl(@ldims) under
    broadcasting: a 1-dim x of dims (n) is accepted against lower dims
    (n, 1) only when n == 1; one lower dim is a scalar every dim is
    compared with; unequal lengths above 1 are a broadcast error."""
    base = str(tmp_path / "m")
    P.writefraw(P.pdl(np.zeros((2, 1, 3))), base)           # dims (3, 1, 2): lower (3, 1)
    with pytest.raises(P.PDLError, match="incompatible lower dims"):
        P.gluefraw(P.pdl(np.zeros(3)), base)                 # (3) vs (3 1): 3 != 1
    P.gluefraw(P.pdl(np.zeros((1, 3))), base)                # (3 1) vs (3 1)
    ones = str(tmp_path / "ones")
    P.writefraw(P.pdl(np.zeros((2, 1, 1))), ones)            # lower dims (1, 1)
    P.gluefraw(P.pdl(np.zeros(1)), ones)                     # (1) broadcasts over (1 1)
    col = str(tmp_path / "col")
    P.writefraw(P.pdl(np.zeros((2, 4))), col)                # lower dims (4): a scalar 4
    with pytest.raises(P.PDLError, match="incompatible lower dims"):
        P.gluefraw(P.pdl(np.zeros((2, 4))), col)             # (4 2): 2 != 4
    P.gluefraw(P.pdl(np.zeros(4)), col)
    cube = str(tmp_path / "cube")
    P.writefraw(P.pdl(np.zeros((2, 4, 3, 2))), cube)         # lower dims (2, 3, 4)
    with pytest.raises(P.PDLError, match="Mismatched implicit broadcast dimension 0: size 2 vs. 3"):
        P.gluefraw(P.pdl(np.zeros((3, 2))), cube)


# ---- files written by the reference PDL's own writefraw
# (tests/golden/make_fraw_fixtures.py; the bytes and headers are PDL's)
GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden" / "fraw"
F32_BAD = np.float32(-3.4028234663852886e38)


def pdl_written():
    """name -> (type, PDL dims, the values PDL wrote, header file or None)"""
    fb = (np.arange(12, dtype=np.float32) / 4).reshape(2, 6)
    fb[0, 1] = F32_BAD
    fb[1, 4] = F32_BAD
    return {
        "seq_double": ("double", (5, 4, 3), np.arange(60, dtype=np.float64).reshape(3, 4, 5) * 1.5 - 7, None),
        "seq_long": ("long", (7, 2), (np.arange(14, dtype=np.int32) * -3).reshape(2, 7), None),
        "seq_byte": ("byte", (9,), np.arange(9, dtype=np.uint8), None),
        "float_bad": ("float", (6, 2), fb, None),
        "own_header": ("double", (3, 2), np.arange(6, dtype=np.float64).reshape(2, 3), "own_header.h"),
    }


@pytest.mark.parametrize("name", sorted(pdl_written()))
def test_reads_files_pdl_wrote(name):
    t, dims, want, hdr = pdl_written()[name]
    y = P.readfraw(str(GOLDEN / name), header=str(GOLDEN / hdr) if hdr else None)
    assert y.type == t and y.dims == dims
    assert y.numpy().tobytes() == want.tobytes()
    m = P.mapfraw(str(GOLDEN / name), ReadOnly=True, Header=str(GOLDEN / hdr) if hdr else None)
    assert m.type == t and m.dims == dims and m.numpy().tobytes() == want.tobytes()


def test_our_writer_matches_pdls_bytes(tmp_path):
    for name, (t, dims, want, hdr) in pdl_written().items():
        if hdr:
            continue
        P.writefraw(P.pdl(want), str(tmp_path / name))
        assert (tmp_path / name).read_bytes() == (GOLDEN / name).read_bytes()
        assert (tmp_path / (name + ".hdr")).read_text() == (GOLDEN / (name + ".hdr")).read_text()


def test_mapfraw_creat_trunc_and_readonly(tmp_path):
    name = str(tmp_path / "m")
    x = P.mapfraw(name, Dims=[4, 3], Datatype=4, Creat=True)   # long->enum
    assert (tmp_path / "m").stat().st_size == 4 * 3 * 4
    assert (tmp_path / "m.hdr").read_text() == "4\n2\n4 3\n"        # long = 4 in PDL's order
    assert x.type == "long" and np.all(x.numpy() == 0)
    # the map is the file: bytes written to the file show through
    with open(name, "r+b") as f:
        f.write(np.arange(12, dtype=np.int32).tobytes())
    assert np.array_equal(x.numpy().reshape(-1), np.arange(12))
    # a header-described map; Trunc zero-fills
    y = P.mapfraw(name, Trunc=True)
    assert y.dims == (4, 3) and np.all(y.numpy() == 0)
    # Datatype defaults to double
    z = P.mapfraw(str(tmp_path / "d"), Dims=[5], Creat=True)
    assert z.type == "double" and (tmp_path / "d").stat().st_size == 40
    # read-only: refused as an op's output, as PDL refuses a read-only output
    r = P.mapfraw(name, ReadOnly=True)
    with pytest.raises(P.PDLError, match=r"PDL::Ufunc::sumover error: output parameter b is read-only"):
        P.sumover(P.pdl(np.ones((3, 4, 5), np.int32)), out=r)
    with pytest.raises(P.PDLError, match="opening file"):
        P.mapfraw(str(tmp_path / "missing"), Dims=[2], ReadOnly=True)
    with pytest.raises(P.PDLError, match="needs 80"):
        P.mapfraw(str(tmp_path / "d"), Dims=[10])
