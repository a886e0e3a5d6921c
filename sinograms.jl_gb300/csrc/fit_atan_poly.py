"""Coefficients of the arc-detector angle polynomials used by the 2D fan back-projector.

atan(q) ~ q * P(q^2) on |q| <= 1 (P of degree 8) and on |q| <= 0.6 (degree 5, for detectors within
+-31 deg): minimax in absolute error, found by Lawson's
iteratively reweighted least squares (C. L. Lawson, 1961) from a least-squares start on a dense
grid.  Running this prints the coefficients as they appear in `sgb_back.cu` and the float32
Horner error against numpy's double atan (about 1.1e-7 rad, i.e. 1e-4 detector bins at
dsd/ds = 927)."""
import numpy as np


def fit(qmax: float = 1.0, n: int = 9, iters: int = 60) -> np.ndarray:
    q = np.linspace(0.0, qmax, 20001)[1:]
    t = q * q
    y = np.arctan(q)
    V = np.stack([q * t ** k for k in range(n)], 1)
    w = np.ones_like(q)
    c = None
    for _ in range(iters):
        c, *_ = np.linalg.lstsq(V * np.sqrt(w)[:, None], y * np.sqrt(w), rcond=None)
        e = np.abs(V @ c - y)
        w = w * e / np.sum(w * e) * len(q)
    return c


def horner_f32(c: np.ndarray, q: np.ndarray) -> np.ndarray:
    q = q.astype(np.float32)
    t = q * q
    p = np.float32(c[-1])
    for k in range(len(c) - 2, -1, -1):
        p = (p * t + np.float32(c[k])).astype(np.float32)
    return p * q


if __name__ == "__main__":
    # atan_poly (|q| <= 1, 9 terms, 1.1e-7 rad) and atan_poly6 (|q| <= 0.6, 6 terms, 8.0e-8 rad)
    for qmax, n in ((1.0, 9), (0.6, 6)):
        c = fit(qmax, n)
        print(f"|q| <= {qmax}, {n} terms:")
        for k, v in enumerate(c):
            print(f"  c{k} = {np.float32(v)!r}")
        q = np.linspace(-qmax, qmax, 400001)
        print("  max abs error (float32 Horner):", float(np.max(np.abs(horner_f32(c, q) - np.arctan(q)))))
