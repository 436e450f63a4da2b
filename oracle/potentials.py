"""ORACLE (test infrastructure only): numpy restatement of ``gaussian_potential``.

Follows mocat/src/utils.py:49-105: the normalising term (d log 2pi - log det_prec)/2
is added only when ``det_prec`` is given or derivable from a diagonal
(1-D) precision / sqrt-precision; the vectorised branch evaluates
0.5 |(x - mean) @ sqrt_prec|^2 (``_vectorised_gaussian_potential`` :25-30), the
diagonal branch 0.5 sum((x - mean)^2 prec) (:41-46), the single full-precision
branch 0.5 (x-m)' prec (x-m) (:33-38).
"""
import warnings

import numpy as np


def gaussian_potential(x, mean=0.0, prec=None, sqrt_prec=None, det_prec=None):
    x = np.atleast_1d(np.asarray(x, np.float64))
    d = x.shape[-1]
    if prec is None and sqrt_prec is None:
        prec = 1.0
    if prec is not None and np.ndim(prec) == 0:
        prec = np.ones(d) * float(prec)
    if sqrt_prec is not None and np.ndim(sqrt_prec) == 0:
        sqrt_prec = np.ones(d) * float(sqrt_prec)
    prec = None if prec is None else np.asarray(prec, np.float64)
    sqrt_prec = None if sqrt_prec is None else np.asarray(sqrt_prec, np.float64)
    if det_prec is None:
        if prec is not None and prec.ndim < 2:
            det_prec = np.prod(prec)
        elif sqrt_prec is not None and sqrt_prec.ndim < 2:
            det_prec = np.prod(sqrt_prec) ** 2
    if det_prec is None:
        neg_log_z = 0.0
        warnings.warn("gaussian_potential: full precision without det_prec -> no normalising constant")
    else:
        neg_log_z = (d * np.log(2 * np.pi) - np.log(det_prec)) / 2
    diff = x - mean
    if x.ndim == 1 and sqrt_prec is None:
        if prec.ndim < 2:
            out = 0.5 * np.sum(diff ** 2 * prec, axis=-1)
        else:
            out = 0.5 * diff @ prec @ diff
    else:
        if prec is not None and sqrt_prec is None:
            sqrt_prec = np.sqrt(prec) if prec.ndim < 2 else np.linalg.cholesky(prec)
        if sqrt_prec.ndim < 2:
            out = 0.5 * np.sum(diff ** 2 * sqrt_prec ** 2, axis=-1)
        else:
            out = 0.5 * np.sum((diff @ sqrt_prec) ** 2, axis=-1)
    return out + neg_log_z
