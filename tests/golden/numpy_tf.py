"""A numpy implementation of the TensorFlow 1.x ops that the reference's
descriptor, pair-term and network-graph functions call
(TFDescriptors/RawSymFunc.py, TFNetworks/TFBehlerParinelloSymEE.py), so that
the golden-fixture scripts beside this file can run those functions
unchanged where TensorFlow is absent. Each op does what the TF op of that
name does for the shapes those functions use: eager, FP64, no graph.
Used only by the fixture generators, never at test time.
"""
from __future__ import annotations

import contextlib

import numpy as np
import scipy.special

# Graph building: the open name scopes, and the values that tf.Variable and a
# model's weight factory hand out, keyed by "scope/.../name"
SCOPE = []
VARIABLES = {}


def scoped(name):
    return "/".join(SCOPE + [name])


class SparseTensor:
    def __init__(self, indices, values, dense_shape):
        self.indices = np.asarray(indices, dtype=np.int64)
        self.values = np.asarray(values)
        self.dense_shape = [int(d) for d in dense_shape]


class _Shape:
    def __init__(self, shape):
        self._shape = list(shape)

    def as_list(self):
        return list(self._shape)


class Tensor(np.ndarray):
    """An ndarray with the static-shape query of a TF tensor."""

    def get_shape(self):
        return _Shape(self.shape)


def constant_tensor(a, dtype=None):
    return np.asarray(a, dtype=dtype).view(Tensor)


class _NN:
    @staticmethod
    def relu(x):
        return np.maximum(x, 0.0)

    @staticmethod
    def dropout(x, keep_prob):
        assert float(keep_prob) == 1.0, "evaluation runs with keep = 1"
        return x


class _GraphKeys:
    TRAINABLE_VARIABLES = "trainable_variables"


class tf:
    float64, float32, int64, int32, bool = np.float64, np.float32, np.int64, np.int32, np.bool_
    SparseTensor = SparseTensor
    nn = _NN
    GraphKeys = _GraphKeys
    matmul = staticmethod(np.matmul)
    add = staticmethod(np.add)
    subtract = staticmethod(np.subtract)
    log = staticmethod(np.log)
    div = staticmethod(np.floor_divide)   # TF 1.x integer division

    @staticmethod
    @contextlib.contextmanager
    def name_scope(name):
        SCOPE.append(name)
        try:
            yield name
        finally:
            SCOPE.pop()

    @staticmethod
    def Variable(initial, trainable=True, dtype=None, name=None):
        if name is not None and scoped(name) in VARIABLES:
            return VARIABLES[scoped(name)]
        return np.asarray(initial, dtype=dtype)

    @staticmethod
    def zeros(shape, dtype=np.float64):
        return np.zeros([int(s) for s in shape], dtype=dtype)

    @staticmethod
    def verify_tensor_all_finite(x, msg):
        assert np.all(np.isfinite(x)), msg
        return x

    @staticmethod
    def cond(pred, f1, f2):
        return f1() if bool(pred) else f2()

    @staticmethod
    def get_collection(key, scope=None):
        return []

    @staticmethod
    def shape(x):
        return np.array(np.shape(x), dtype=np.int64)

    sqrt = staticmethod(np.sqrt)
    exp = staticmethod(np.exp)
    cos = staticmethod(np.cos)
    acos = staticmethod(np.arccos)
    multiply = staticmethod(np.multiply)
    pow = staticmethod(np.power)
    greater = staticmethod(np.greater)
    greater_equal = staticmethod(np.greater_equal)
    less_equal = staticmethod(np.less_equal)
    is_nan = staticmethod(np.isnan)
    erfc = staticmethod(scipy.special.erfc)

    @staticmethod
    def equal(a, b, name=None):
        return np.equal(a, b)

    @staticmethod
    def zeros_like(x, dtype=None):
        return np.zeros_like(x, dtype=dtype)

    @staticmethod
    def ones_like(x, dtype=None):
        return np.ones_like(x, dtype=dtype)

    @staticmethod
    def reduce_sum(x, axis=None):
        return np.sum(x, axis=axis)

    @staticmethod
    def reduce_max(x, axis=None):
        return np.max(x, axis=axis)

    @staticmethod
    def constant(v, dtype=None):
        return np.array(v, dtype=dtype)

    @staticmethod
    def cast(x, dtype, name=None):
        return np.asarray(x).astype(dtype)

    @staticmethod
    def reshape(x, shape, name=None):
        return np.reshape(x, [int(s) for s in shape])

    @staticmethod
    def range(n, dtype=np.int32):
        return np.arange(int(n), dtype=dtype)

    @staticmethod
    def stack(xs, axis=0):
        return np.stack(xs, axis)

    @staticmethod
    def concat(xs, axis, name=None):
        return np.concatenate(xs, axis)

    @staticmethod
    def tile(x, reps):
        return np.tile(x, [int(r) for r in reps])

    @staticmethod
    def transpose(x, perm):
        return np.transpose(x, perm)

    @staticmethod
    def expand_dims(x, axis):
        return np.expand_dims(x, axis)

    @staticmethod
    def slice(x, begin, size):
        sl = tuple(slice(int(b), None if int(s) == -1 else int(b) + int(s)) for b, s in zip(begin, size))
        return np.asarray(x)[sl]

    @staticmethod
    def gather_nd(params, indices):
        idx = np.asarray(indices).astype(np.int64)
        return np.asarray(params)[tuple(idx[..., k] for k in range(idx.shape[-1]))]

    @staticmethod
    def scatter_nd(indices, updates, shape):
        """Sums updates that land on the same index, as tf.scatter_nd does."""
        out = np.zeros([int(s) for s in shape], dtype=np.asarray(updates).dtype)
        idx = np.asarray(indices).astype(np.int64)
        np.add.at(out, tuple(idx[..., k] for k in range(idx.shape[-1])), updates)
        return out

    @staticmethod
    def boolean_mask(x, mask):
        return np.asarray(x)[np.asarray(mask, dtype=bool)]

    @staticmethod
    def where(cond, x=None, y=None):
        if x is None:
            return np.argwhere(cond).astype(np.int64)   # row-major, as tf.where
        return np.where(cond, x, y)

    @staticmethod
    def sparse_reduce_sum(sp, axis):
        assert axis == 1
        out = np.zeros(sp.dense_shape[0], dtype=sp.values.dtype)
        np.add.at(out, sp.indices[:, 0], sp.values)
        return out
