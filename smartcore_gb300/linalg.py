"""DenseMatrix: the data container the estimators take.

Mirrors smartcore's DenseMatrix (src/linalg/basic/matrix.rs:24-32, :187-238):
a shape, a flat value vector and a column_major flag, column-major by default
(from_2d_array / from_2d_vec build column-major storage).  Any 2-D numpy
array is accepted by the estimators as well; its memory order is passed to
the C ABI as-is (SC_ROW_MAJOR / SC_COL_MAJOR), with no host transpose.
"""
from __future__ import annotations

import numpy as np

from .error import Failed, FailedError


class DenseMatrix:
    def __init__(self, nrows, ncols, values, column_major=True, dtype=None):
        values = np.asarray(values, dtype=dtype)
        if nrows * ncols != values.size:
            raise Failed(FailedError.ParametersError,
                         f"The specified shape: (cols: {ncols}, rows: {nrows}) does not align "
                         f"with data len: {values.size}")
        self.nrows, self.ncols, self.column_major = nrows, ncols, column_major
        flat = values.reshape(-1)
        self._a = (flat.reshape(ncols, nrows).T if column_major else flat.reshape(nrows, ncols))

    @staticmethod
    def new(nrows, ncols, values, column_major, dtype=None):
        return DenseMatrix(nrows, ncols, values, column_major, dtype)

    @staticmethod
    def from_2d_array(rows, dtype=np.float64):
        if len(rows) == 0 or len(rows[0]) == 0:
            raise Failed(FailedError.ParametersError,
                         "The 2d vec provided is empty; cannot instantiate the matrix")
        a = np.asarray(rows, dtype=dtype)
        return DenseMatrix(a.shape[0], a.shape[1], a.T.reshape(-1), True)

    from_2d_vec = from_2d_array

    def shape(self):
        return (self.nrows, self.ncols)

    def get(self, pos):
        return self._a[pos]

    def array(self):
        """The values as a 2-D numpy view (Fortran order when column-major)."""
        return self._a


def as_matrix(x, dtype=None):
    """2-D float32/float64 array view of x (DenseMatrix or array-like),
    keeping C or Fortran order when possible."""
    a = x.array() if isinstance(x, DenseMatrix) else np.asarray(x)
    if a.ndim == 1:
        a = a[:, None]
    if dtype is not None and a.dtype != dtype:
        a = a.astype(dtype, order="K")
    elif a.dtype not in (np.float32, np.float64):
        a = a.astype(np.float64, order="K")
    if not (a.flags.c_contiguous or a.flags.f_contiguous):
        a = np.ascontiguousarray(a)
    return a


def layout_of(a):
    """(layout code, leading dimension) of a contiguous 2-D array."""
    if a.flags.c_contiguous:
        return 0, a.shape[1]
    return 1, a.shape[0]
