"""f32 transforms with the reference's arithmetic (src/transform/*.rs).

All arithmetic uses numpy float32 scalars one operation at a time, in the
order the Rust source writes it, so results are the crate's bit for bit
(numpy scalar float32 ops are single IEEE operations; no FMA).
"""
from __future__ import annotations

import numpy as np

from . import abi

F = np.float32
ZERO, ONE = F(0.0), F(1.0)


def _mat(rows) -> np.ndarray:
    return np.array(rows, dtype=np.float32).reshape(4, 4)


def identity() -> np.ndarray:
    return np.eye(4, dtype=np.float32)


def mat_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """src/transform/matrix4x4.rs:167-182 (left-to-right sums)."""
    r = np.zeros((4, 4), dtype=np.float32)
    for i in range(4):
        for j in range(4):
            r[i, j] = a[i, 0] * b[0, j] + a[i, 1] * b[1, j] + a[i, 2] * b[2, j] + a[i, 3] * b[3, j]
    return r


def mat_inverse(a: np.ndarray) -> np.ndarray:
    """src/transform/matrix4x4.rs:66-160: scaled partial pivoting (row swaps
    exchange columns k..3 only), then one solve per unit vector."""
    lu = a.astype(np.float32).copy()
    scale = []
    for i in range(4):
        s = ZERO
        for j in range(4):
            s = np.fmax(abs(lu[i, j]), s)
        scale.append(F(s))
    piv = [0, 1, 2, 3]
    for k in range(3):
        best, p = ZERO, k
        for i in range(k, 4):
            c = abs(lu[i, k] / scale[i])
            if c > best:
                best, p = c, i
        piv[k] = p
        if best == ZERO:
            raise ValueError("Singular matrix!")
        if p != k:
            for j in range(k, 4):
                lu[k, j], lu[p, j] = lu[p, j], lu[k, j]
        for i in range(k + 1, 4):
            f = lu[i, k] / lu[k, k]
            lu[i, k] = f
            for j in range(k + 1, 4):
                lu[i, j] = lu[i, j] - f * lu[k, j]
    if abs(lu[3, 3]) < F(1.0e-6):
        raise ValueError("Singular matrix!")
    inv = np.zeros((4, 4), dtype=np.float32)
    for c in range(4):
        x = [ZERO, ZERO, ZERO, ZERO]
        x[c] = ONE
        for k in range(3):
            if piv[k] != k:
                x[piv[k]], x[k] = x[k], x[piv[k]]
            for i in range(k + 1, 4):
                x[i] = F(x[i] - lu[i, k] * x[k])
        x[3] = F(x[3] / lu[3, 3])
        for i in range(2, -1, -1):
            acc = ZERO
            for j in range(i + 1, 4):
                acc = F(acc + lu[i, j] * x[j])
            x[i] = F((x[i] - acc) / lu[i, i])
        for r in range(4):
            inv[r, c] = x[r]
    return inv


_libm = None


def _libm_f(name: str):
    """The C library's f32 function (what Rust's f32 methods call on Linux)."""
    global _libm
    import ctypes
    import ctypes.util
    if _libm is None:
        _libm = ctypes.CDLL(ctypes.util.find_library("m") or None)
    fn = getattr(_libm, name)
    fn.restype, fn.argtypes = ctypes.c_float, [ctypes.c_float]
    return fn


def _sinf(x) -> np.float32:
    return F(_libm_f("sinf")(float(x)))


def _cosf(x) -> np.float32:
    return F(_libm_f("cosf")(float(x)))


def _as_radians(deg) -> np.float32:
    """utils/mod.rs: degrees * pi / 180 in f32."""
    return F(F(F(deg) * F(np.pi)) / F(180.0))


def _v(x) -> tuple:
    return tuple(F(c) for c in x)


def _normalize(v) -> tuple:
    x, y, z = v
    ln = np.sqrt(F(x * x + y * y + z * z))
    r = ONE / ln
    return (F(x * r), F(y * r), F(z * r))


def _cross(a, b) -> tuple:
    return (F(a[1] * b[2] - a[2] * b[1]), F(a[2] * b[0] - a[0] * b[2]), F(a[0] * b[1] - a[1] * b[0]))


class Transform:
    """The reference Transform {m, m_inv} (src/transform/transform.rs:14-19)."""

    __slots__ = ("m", "m_inv")

    def __init__(self, m: np.ndarray | None = None, m_inv: np.ndarray | None = None):
        self.m = identity() if m is None else np.asarray(m, dtype=np.float32).reshape(4, 4).copy()
        self.m_inv = identity() if m_inv is None else np.asarray(m_inv, dtype=np.float32).reshape(4, 4).copy()

    @staticmethod
    def from_matrix(m) -> "Transform":
        """transform.rs:288-293: the inverse comes from the reference LU."""
        m = np.asarray(m, dtype=np.float32).reshape(4, 4)
        return Transform(m, mat_inverse(m))

    @staticmethod
    def translate(v) -> "Transform":
        """transform.rs:39-51."""
        x, y, z = _v(v)
        m = _mat([[1, 0, 0, x], [0, 1, 0, y], [0, 0, 1, z], [0, 0, 0, 1]])
        mi = _mat([[1, 0, 0, -x], [0, 1, 0, -y], [0, 0, 1, -z], [0, 0, 0, 1]])
        return Transform(m, mi)

    @staticmethod
    def scale(x, y, z) -> "Transform":
        """transform.rs:53-65."""
        x, y, z = F(x), F(y), F(z)
        m = _mat([[x, 0, 0, 0], [0, y, 0, 0], [0, 0, z, 0], [0, 0, 0, 1]])
        mi = _mat([[ONE / x, 0, 0, 0], [0, ONE / y, 0, 0], [0, 0, ONE / z, 0], [0, 0, 0, 1]])
        return Transform(m, mi)

    @staticmethod
    def look_at(pos, look, up) -> "Transform":
        """transform.rs:144-174: returns world-to-camera = Transform(inv(m), m)."""
        pos, look, up = _v(pos), _v(look), _v(up)
        d = _normalize((F(look[0] - pos[0]), F(look[1] - pos[1]), F(look[2] - pos[2])))
        left = _normalize(_cross(_normalize(up), d))
        new_up = _cross(d, left)
        m = identity()
        m[0, 3], m[1, 3], m[2, 3], m[3, 3] = pos[0], pos[1], pos[2], ONE
        m[0, 0], m[1, 0], m[2, 0], m[3, 0] = left[0], left[1], left[2], ZERO
        m[0, 1], m[1, 1], m[2, 1], m[3, 1] = new_up[0], new_up[1], new_up[2], ZERO
        m[0, 2], m[1, 2], m[2, 2], m[3, 2] = d[0], d[1], d[2], ZERO
        return Transform(mat_inverse(m), m)

    @staticmethod
    def rotate(angle, axis) -> "Transform":
        """transform.rs:117-142 (the inverse is the transpose)."""
        a = _normalize(_v(axis))
        th = _as_radians(angle)
        s, c = _sinf(th), _cosf(th)
        ax, ay, az = a
        one_c = F(ONE - c)
        m = identity()
        m[0, 0] = F(ax * ax + F(F(ONE - F(ax * ax)) * c))
        m[0, 1] = F(F(F(ax * ay) * one_c) - F(az * s))
        m[0, 2] = F(F(F(ax * az) * one_c) + F(ay * s))
        m[1, 0] = F(F(F(ax * ay) * one_c) + F(az * s))
        m[1, 1] = F(ay * ay + F(F(ONE - F(ay * ay)) * c))
        m[1, 2] = F(F(F(ay * az) * one_c) - F(ax * s))
        m[2, 0] = F(F(F(ax * az) * one_c) - F(ay * s))
        m[2, 1] = F(F(F(ay * az) * one_c) + F(ax * s))
        m[2, 2] = F(az * az + F(F(ONE - F(az * az)) * c))
        return Transform(m, m.T.copy())

    def inverse(self) -> "Transform":
        return Transform(self.m_inv, self.m)

    def __mul__(self, other: "Transform") -> "Transform":
        """transform.rs:266-271."""
        return Transform(mat_mul(self.m, other.m), mat_mul(other.m_inv, self.m_inv))

    def __eq__(self, other) -> bool:
        return isinstance(other, Transform) and np.array_equal(self.m, other.m) and np.array_equal(
            self.m_inv, other.m_inv)

    def point(self, p) -> tuple:
        """transform.rs:195-208."""
        m = self.m
        x, y, z = _v(p)
        xt = m[0, 0] * x + m[0, 1] * y + m[0, 2] * z + m[0, 3]
        yt = m[1, 0] * x + m[1, 1] * y + m[1, 2] * z + m[1, 3]
        zt = m[2, 0] * x + m[2, 1] * y + m[2, 2] * z + m[2, 3]
        w = m[3, 0] * x + m[3, 1] * y + m[3, 2] * z + m[3, 3]
        if w != ONE:
            return (F(xt / w), F(yt / w), F(zt / w))
        return (F(xt), F(yt), F(zt))

    def vector(self, v) -> tuple:
        """transform.rs:210-218."""
        m = self.m
        x, y, z = _v(v)
        return (F(m[0, 0] * x + m[0, 1] * y + m[0, 2] * z), F(m[1, 0] * x + m[1, 1] * y + m[1, 2] * z),
                F(m[2, 0] * x + m[2, 1] * y + m[2, 2] * z))

    def to_abi(self) -> abi.PbrtTransform:
        t = abi.PbrtTransform()
        t.m[:] = [float(x) for x in self.m.reshape(-1)]
        t.m_inv[:] = [float(x) for x in self.m_inv.reshape(-1)]
        return t

