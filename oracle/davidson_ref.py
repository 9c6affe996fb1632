"""Line-by-line CPU restatement of ``src/davidson.rs`` -- TEST INFRASTRUCTURE ONLY.

Follows ``davidson_solve`` (davidson.rs:48-266) and its helpers
``_normalize_xt_`` (:268-285), ``_qr`` (:287-325), ``fill_heff`` (:327-390),
``_gen_x0`` (:392-404) and ``_sort_elast`` (:406-432), keeping the reference's
quirks:

* the preconditioner shifts every root by ``e[0]`` (:224);
* ``_sort_elast`` computes an overlap reordering but returns its inputs (:406-432);
* ``max_dx_last`` is shadowed at the end of each cycle, so the restart test
  (:210) always compares against the value set at the last fresh start (1e9);
* ``maxspace += 3 (nroots - 1)`` (:74); ``tol_res`` is unused (:61);
* the Rayleigh-Ritz step packs the upper triangle and calls ``dspevx`` with
  range 'A' and abstol 1e-16 (matrix_blas_lapack.rs:1075-1095);
* in the non-fresh branch ``xtlen`` is taken before ``_qr`` (:112-118).

``_qr`` also forms R^-1 through dgetrf/dgetri, which every caller discards
(``.0``); that inverse is not formed here.  Vector norms and dot products are
plain float64 sums (nalgebra ``DVector::norm``/``dot``).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, List, Tuple

import numpy as np


@dataclass
class DavidsonParams:
    """davidson.rs:28-46 (defaults at :36-46)."""

    tol: float = 1e-5
    maxcyc: int = 50
    maxspace: int = 12
    lindep: float = 1e-14
    nroots: int = 3


def _normalize_xt_(xt: List[np.ndarray], lindep: float) -> Tuple[List[np.ndarray], float]:
    norm_min = 1.0
    out = []
    for x in xt:
        norm = float(np.linalg.norm(x))
        if norm ** 2 > lindep:
            out.append(x / norm)
            norm_min = min(norm_min, norm)
    return out, norm_min


def _qr(x: List[np.ndarray], lindep: float) -> List[np.ndarray]:
    """Modified Gram-Schmidt (davidson.rs:287-325); returns the kept q vectors."""
    qs: List[np.ndarray] = []
    for xi0 in x:
        xi = xi0.copy()
        for q in qs:
            prod = float(np.dot(q, xi))
            xi -= q * prod
        norm = float(np.linalg.norm(xi))
        if norm ** 2 > lindep:
            qs.append(xi / norm)
    return qs


def fill_heff(heff_old: np.ndarray, xs, ax, xtlen: int, fresh_start: bool) -> np.ndarray:
    """davidson.rs:327-390; heff is symmetric, so its storage order is immaterial."""
    row1 = len(ax)
    row0 = row1 - xtlen
    space = row1
    heff = np.zeros((space, space))
    if not fresh_start:
        so = heff_old.shape[0]
        heff[:so, :so] = heff_old
    for i in range(row0, row1):
        for j in range(row0, row1):
            v = float(np.dot(xs[i], ax[j]))
            heff[i, j] = v
            heff[j, i] = v
    for j in range(row0, row1):
        for i in range(0, row0):
            v = float(np.dot(ax[i], xs[j]))
            heff[i, j] = v
            heff[j, i] = v
    return heff


def _gen_x0(v: np.ndarray, x) -> List[np.ndarray]:
    """X * V through dgemm (davidson.rs:392-404)."""
    from . import dgemm

    xmat = np.asfortranarray(np.stack(x, axis=1))
    x0 = dgemm("N", "N", xmat, v)
    return [x0[:, k].copy() for k in range(x0.shape[1])]


def davidson_solve(a_x: Callable[[np.ndarray], np.ndarray], x0_1d: np.ndarray, hdiag: np.ndarray,
                   params: DavidsonParams, print_level: int = 0):
    """Returns (conv, e, x0) like davidson.rs:48-266."""
    from . import dspevx_packed, full_to_upper_packed

    tol, maxcyc, lindep, nroots = params.tol, params.maxcyc, params.lindep, params.nroots
    maxspace = params.maxspace + (nroots - 1) * 3
    hdiag = np.asarray(hdiag, dtype=np.float64)

    def precond(dx, e):
        hd = hdiag - e
        hd = np.where(np.abs(hd) < 1e-8, 1e-8, hd)
        return dx / hd

    x0 = [np.array(x0_1d, dtype=np.float64)]
    fresh_start = True
    xt: List[np.ndarray] = []
    xtlen = 0
    xs: List[np.ndarray] = []
    ax: List[np.ndarray] = []
    space = 0
    ov = len(x0_1d)
    e: List[float] = []
    v = np.zeros((0, 0))
    conv = [False] * nroots
    max_dx_last = 1e9
    heff = np.zeros((0, 0))
    nroots_current = 0
    for icyc in range(maxcyc):
        if fresh_start:
            xs, ax, space = [], [], 0
            xt = _qr(x0, lindep)
            xtlen = len(xt)
            if ov - nroots < 3:
                raise RuntimeError("Too much nroots required")
            if xtlen == 0:
                raise RuntimeError("No more linear independent basis found")
            max_dx_last = 1e9
        else:
            xtlen = len(xt)
            if xtlen > 1:
                xt = _qr(list(xt), lindep)
                if xtlen > 40:
                    xt = xt[:40]
        for xi in xt:
            axi = np.asarray(a_x(xi.copy()), dtype=np.float64)
            xs.append(xi.copy())
            ax.append(axi.copy())
        head = space
        space = space + xtlen
        elast = list(e)
        vlast = v.copy()
        convlast = list(conv)
        heff = fill_heff(heff, xs, ax, xtlen, fresh_start)
        eigvec, eigval, _nf = dspevx_packed(full_to_upper_packed(heff))
        if len(eigval) < nroots:
            e = list(eigval)
            v = np.asfortranarray(eigvec)
        else:
            e = list(eigval[:nroots])
            v = np.asfortranarray(eigvec[:space, :nroots])
        nroots_current = min(len(eigval), nroots)
        x0 = _gen_x0(v, xs)
        ax0 = _gen_x0(v, ax)
        # _sort_elast returns (elast, convlast) unchanged in every branch.
        xt = []
        dx_norm = [0.0] * nroots_current
        de = [0.0] * nroots_current
        for k in range(nroots_current):
            de[k] = e[k] - elast[k] if k < len(elast) else e[k]
            xt_k = ax0[k] - e[k] * x0[k]
            xt.append(xt_k)
            dx_norm[k] = float(np.linalg.norm(xt_k))
            conv[k] = abs(de[k]) < tol and dx_norm[k] < np.sqrt(tol)
        all_conv = all(conv)
        max_dx_norm = max(dx_norm)
        if all_conv:
            break
        if max_dx_norm > 1.0 and max_dx_norm / max_dx_last > 3.0 and space > nroots + 2:
            x0 = _gen_x0(vlast, xs)
            fresh_start = True
            continue
        xt_new = []
        for k in range(nroots_current):
            if dx_norm[k] ** 2 > lindep:
                t = precond(xt[k], e[0])
                t = t / float(np.linalg.norm(t))
                xt_new.append(t)
        xt = xt_new
        for i in range(space):
            for k in range(len(xt)):
                xt[k] = xt[k] - xs[i] * float(np.dot(xs[i], xt[k]))
        xt, _norm_min = _normalize_xt_(xt, lindep)
        if len(xt) == 0:
            for k in range(len(dx_norm)):
                conv[k] = conv[k] or dx_norm[k] < np.sqrt(tol)
            break
        fresh_start = space + nroots > maxspace
        del head
    return conv, e, x0
