"""PDL::IO::FastRaw (lib/PDL/IO/FastRaw.pm:198-350): an ndarray's bytes in
one file and a text header beside it ("<name>.hdr" unless `header` names
another file: type id, ndims, dims).  readfraw(device=True) copies the
file into device memory from a mapping of it (a file that cannot be mapped
streams through pinned staging buffers, the reads overlapping the copies),
so no copy of the data is made in process memory."""
from __future__ import annotations

import ctypes as C
import importlib
import mmap
import os
from typing import Optional

import numpy as np

from . import _abi as A
from ._abi import PDLError, check, lib

N = importlib.import_module(".ndarray", __package__)


def _enc(s: Optional[str]):
    return None if s is None else os.fsencode(s)


def read_header(name: str, header: Optional[str] = None):
    """(type code, dims) from a FastRaw header (_read_frawhdr)."""
    d = A.Ndarray()
    check(lib().pdlgb300_fraw_header(_enc(name), _enc(header), C.byref(d)))
    return d.datatype, tuple(d.dims[i] for i in range(d.ndims))


def readfraw(name: str, header: Optional[str] = None, device: bool = False) -> "N.ndarray":
    """The ndarray in `name` (readfraw); device=True puts it in device memory."""
    t, dims = read_header(name, header)
    n = int(np.prod(dims, dtype=np.int64)) if dims else 1
    if device:
        x = N.device_empty(t, *dims)
    else:
        nbytes = n * np.dtype(N.NP_DTYPES[t]).itemsize
        x = N.ndarray(N.Storage(nbytes, host=np.zeros(max(nbytes, 1), np.uint8)), t, dims)
    d = x._desc(device)
    check(lib().pdlgb300_readfraw_into(_enc(name), C.byref(d)))
    x.storage.fresh = "dev" if device else "host"
    return x


def _contiguous(x: "N.ndarray") -> "N.ndarray":
    s = 1
    for d, i in zip(x.dims, x.incs):
        if d > 1 and i != s:
            return N.convert(x, x.datatype)
        s *= d
    return x


def writefraw(x: "N.ndarray", name: str, header: Optional[str] = None) -> None:
    """The header and the data of x (writefraw), from host or device memory."""
    x = _contiguous(x)
    d = x._desc(x.on_device)
    check(lib().pdlgb300_writefraw(C.byref(d), _enc(name), _enc(header)))


def _shape_matches(shape, low) -> bool:
    """PDL::all($pdl->shape == pdl(@ldims)) (FastRaw.pm:338-339) under PDL's
    broadcasting: pdl() of one number is a 0-dim scalar that every element of
    the shape is compared with; otherwise two 1-dim ndarrays whose lengths
    must be equal, or one of them 1 (its element compared with every element
    of the other), else the comparison itself dies with a broadcast error.
    The all() of an empty comparison is true."""
    if len(low) == 1:
        return all(d == low[0] for d in shape)
    if len(shape) == len(low):
        return all(d == l for d, l in zip(shape, low))
    if len(shape) == 1:
        return all(shape[0] == l for l in low)
    raise PDLError(A.EUSERERROR,
                   f"Mismatched implicit broadcast dimension 0: size {len(shape)} vs. {len(low)}")


def gluefraw(x: "N.ndarray", name: str, header: Optional[str] = None) -> None:
    """Append x as one more step of the last dim of the file's ndarray
    (gluefraw, FastRaw.pm:326-346), with the reference's checks."""
    if not os.path.isfile(name):
        raise PDLError(A.EUSERERROR, f"'{name}' must be real filename")
    t, dims = read_header(name, header)
    if x.datatype != t:
        raise PDLError(A.EUSERERROR, f"gluefraw: ndarray has type '{x.type}' but file has type '{t}'")
    if len(dims) < 2:
        raise PDLError(A.EUSERERROR, f"gluefraw: header dims needs at least 2 dims, got ({' '.join(map(str, dims))})")
    low = list(dims[:-1])
    if not _shape_matches(list(x.dims), low):
        raise PDLError(A.EUSERERROR,
                       f"gluefraw: incompatible lower dims, ndarray ({' '.join(map(str, x.dims))}) "
                       f"vs header ({' '.join(map(str, low))})")
    with open(name, "ab") as f:
        f.write(np.ascontiguousarray(x.numpy()).tobytes())
    new_dims = list(dims[:-1]) + [dims[-1] + 1]
    hname = header or name + ".hdr"
    with open(hname, "w") as h:
        h.write(f"{t}\n{len(new_dims)}\n{' '.join(map(str, new_dims))}\n")


def mapfraw(name: str, Dims=None, Datatype: Optional[int] = None, Creat: bool = False,
            Trunc: bool = False, ReadOnly: bool = False, Header: Optional[str] = None) -> "N.ndarray":
    """PDL::mapfraw (lib/PDL/IO/FastRaw.pm:393-418): the file mapped as the
    ndarray's host memory (a shared mapping: set_data_by_file_map).  Dims and
    Datatype give the shape instead of the header (Datatype defaults to
    double); Creat creates the file and writes its header; Creat or Trunc
    sizes the file to the data, zero-filled; ReadOnly maps it read-only.

    On the GPU: to_device() copies the mapped bytes into a device mirror;
    results an op writes there reach the file when the ndarray is brought
    back to the host (to_host(), numpy()), because the host memory is the
    mapping.  A read-only map is refused as an op's output, as PDL refuses a
    read-only output."""
    if Dims is not None:
        t = A.D if Datatype is None else int(Datatype)
        dims = tuple(int(d) for d in Dims)
    else:
        t, dims = read_header(name, Header)
    if t not in N.NP_DTYPES:
        raise PDLError(A.EUSERERROR, f"mapfraw: type {t} is not on this path")
    nbytes = int(np.prod(dims, dtype=np.int64)) * np.dtype(N.NP_DTYPES[t]).itemsize if dims \
        else np.dtype(N.NP_DTYPES[t]).itemsize
    flags = os.O_RDONLY if ReadOnly else os.O_RDWR
    if Creat:
        flags |= os.O_CREAT
    try:
        fd = os.open(name, flags, 0o644)
    except OSError as e:
        raise PDLError(A.EUSERERROR, f"Error opening file '{name}': {e.strerror}") from None
    try:
        if Creat or Trunc:
            os.ftruncate(fd, 0)
            os.ftruncate(fd, nbytes)
        size = os.fstat(fd).st_size
        if size < nbytes:
            raise PDLError(A.EUSERERROR, f"mapfraw: '{name}' has {size} bytes, the ndarray needs {nbytes}")
        if nbytes:
            mm = mmap.mmap(fd, nbytes, mmap.MAP_SHARED,
                           mmap.PROT_READ if ReadOnly else mmap.PROT_READ | mmap.PROT_WRITE)
            host = np.frombuffer(mm, dtype=np.uint8)
        else:
            host = np.zeros(1, np.uint8)
    finally:
        os.close(fd)
    st = N.Storage(nbytes, host=host)
    st.readonly = bool(ReadOnly)
    x = N.ndarray(st, t, dims)
    if Creat:
        with open(Header or name + ".hdr", "w") as f:
            f.write(f"{t}\n{len(dims)}\n{' '.join(map(str, dims))}\n")
    return x
