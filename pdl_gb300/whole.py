"""Whole-array reductions (lib/PDL/Ufunc.pd:615-663): each one flattens its
argument (clump(-1), a view where the strides allow) and runs the matching
reduction over dim 0, returning a 0-dim ndarray.  and/or are keywords in
Python, so those two are and_/or_; any/all alias or_/and_ as in the
reference (Ufunc.pd:665-710).  median, oddmedian, mode, pct and oddpct are
the sort-based ones (Ufunc.pd:615-663, 1009-1038)."""
from .ndarray import _scalar_to_pdl


def _whole(method):
    def f(x):
        return getattr(_scalar_to_pdl(x, None), method)()
    f.__name__ = method
    f.__doc__ = f"{method} of all elements (x.flat() then the reduction over dim 0)."
    return f


sum = _whole("sum")  # noqa: A001
avg = _whole("avg")
prod = _whole("prod")
dsum = _whole("dsum")
davg = _whole("davg")
dprod = _whole("dprod")
zcheck = _whole("zcheck")
and_ = _whole("and_")
band = _whole("band")
or_ = _whole("or_")
bor = _whole("bor")
xorall = _whole("xorall")
bxor = _whole("bxor")
min = _whole("min")  # noqa: A001
max = _whole("max")  # noqa: A001
any = or_  # noqa: A001
all = and_  # noqa: A001
median = _whole("median")
oddmedian = _whole("oddmedian")
mode = _whole("mode")


def pct(x, p):
    """The p-th percentile of all elements, interpolated (Ufunc.pd:1009-1038)."""
    return _scalar_to_pdl(x, None).pct(p)


def oddpct(x, p):
    """The p-th percentile of all elements, the nearest data value."""
    return _scalar_to_pdl(x, None).oddpct(p)
