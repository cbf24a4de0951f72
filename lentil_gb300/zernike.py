"""Zernike OPD generators on the GPU, drop-in for lentil's
(lentil/zernike.py:11-234, 348-480).

Coordinates (mask centroid origin, rho = 1 at the farthest masked pixel)
and the polynomial sums run in the library's kernels; the host only turns
mode indices into a small table of (m, scale, radial-polynomial terms) with
lentil's formulas.  numpy arrays in give numpy arrays out; CUDA tensors in
give CUDA tensors out."""
from math import factorial

import numpy as np
import torch

from . import _device as dv
from . import _lib


def noll_to_nm(j):
    """Noll index -> (n, m) (lentil/zernike.py:348-391; Noll 1976 ordering:
    within a radial order, |m| increases, cosine terms take even j)."""
    if j < 1:
        raise ValueError('Noll index must be greater than zero')
    n = 0
    while (n + 1) * (n + 2) // 2 < j:
        n += 1
    first = n * (n + 1) // 2 + 1            # first Noll index of radial order n
    pos = j - first                          # 0-based position inside the order
    ms = [m for m in range(n % 2, n + 1, 2) for _ in ((0,) if m == 0 else (0, 1))]
    m = ms[pos]
    return n, (m if j % 2 == 0 else -m)


def ansi_to_nm(j):
    """ANSI index -> (n, m) (lentil/zernike.py:394-415)."""
    if j < 0:
        raise ValueError('ANSI index must be zero or larger')
    n = int(np.floor((np.sqrt(8 * j + 1) - 1) / 2))
    return n, int(2 * j - n * (n + 2))


def fringe_to_nm(j):
    """Fringe index -> (n, m) (lentil/zernike.py:418-441)."""
    if j < 1:
        raise ValueError('Fringe index must be greater than zero')
    m_n = 2 * (np.ceil(np.sqrt(j)) - 1)
    g_s = (m_n / 2) ** 2 + 1
    n = m_n / 2 + np.floor((j - g_s) / 2)
    m = (m_n - n) * (1 - np.mod(j - g_s, 2) * 2)
    return int(n), int(m)


_ORDERS = {'noll': noll_to_nm, 'fringe': fringe_to_nm, 'ansi': ansi_to_nm}


def _nm(index, order):
    if order not in _ORDERS:
        raise ValueError('Unknown order', order)
    return _ORDERS[order](int(index))


def radial_terms(n, m):
    """(coefficient, power) terms of the radial polynomial R_n^m in lentil's
    summation order (lentil/zernike.py:96-109); empty when n - |m| is odd."""
    m, n = abs(int(m)), abs(int(n))
    if (n - m) & 1:
        return []
    return [((-1) ** k * factorial(n - k) /
             (factorial(k) * factorial((n + m) // 2 - k) * factorial((n - m) // 2 - k)),
             n - 2 * k) for k in range((n - m) // 2 + 1)]


def _mode_table(indices, coeffs, normalize, order):
    """Device table: per mode [m, scale, nterms, (coef, power) x T]."""
    rows = []
    for j, c in zip(indices, coeffs):
        n, m = _nm(j, order)
        if m == 0 and n == 0:
            terms, norm = [(1.0, 0)], 1.0                 # Z_1 is the mask itself
        else:
            terms = radial_terms(n, m)
            if not normalize:
                norm = 1.0
            elif m == 0:
                norm = np.sqrt(n + 1)
            else:
                norm = np.sqrt(2) * np.sqrt(n + 1)
        rows.append((m, float(c) * norm, terms))
    T = max(1, max(len(r[2]) for r in rows))
    tab = np.zeros((len(rows), 3 + 2 * T))
    for k, (m, scale, terms) in enumerate(rows):
        tab[k, 0], tab[k, 1], tab[k, 2] = m, scale, len(terms)
        for t, (a, p) in enumerate(terms):
            tab[k, 3 + 2 * t], tab[k, 4 + 2 * t] = a, p
    return torch.as_tensor(tab, device=dv.device()), len(rows), T


def _mask_device(mask):
    return dv.to_device(mask, torch.float64).contiguous()


def _coords_device(mask_d, shift=None, rotate=0):
    H, W = (int(x) for x in mask_d.shape)
    rho = torch.empty((H, W), dtype=torch.float64, device=mask_d.device)
    theta = torch.empty_like(rho)
    ws = dv.workspace(_lib.load().lgb_zernike_workspace_size())
    auto = shift is None
    sr, sc = (0.0, 0.0) if auto else (float(shift[0]), float(shift[1]))
    _lib.call('lgb_zernike_coordinates', mask_d.data_ptr(), H, W, int(auto), sr, sc,
              float(rotate), rho.data_ptr(), theta.data_ptr(), ws.data_ptr(), ws.numel(),
              dv.stream_ptr())
    return rho, theta


def _out(t, like):
    return t if dv.is_tensor(like) else dv.to_host(t)


def zernike_coordinates(mask, shift=None, rotate=0):
    """(rho, theta) of ``mask``: origin at the mask centroid (or ``shift``
    pixels from the centre), rho = 1 at the farthest masked pixel, theta
    measured from +x (lentil/zernike.py:444-480)."""
    rho, theta = _coords_device(_mask_device(mask), shift, rotate)
    return _out(rho, mask), _out(theta, mask)


def _eval(mask, indices, coeffs, normalize, order, rho, theta, basis):
    mask_d = _mask_device(mask)
    if rho is None:
        rho_d, theta_d = _coords_device(mask_d)
    else:
        if theta is None:
            raise ValueError('Both rho and theta must be specified')
        rho_d = dv.to_device(rho, torch.float64).contiguous()
        theta_d = dv.to_device(theta, torch.float64).contiguous()
    tab, K, T = _mode_table(indices, coeffs, normalize, order)
    shape = tuple(mask_d.shape)
    out = torch.empty(((K,) if basis else ()) + shape, dtype=torch.float64, device=mask_d.device)
    _lib.call('lgb_zernike_eval', rho_d.data_ptr(), theta_d.data_ptr(), mask_d.data_ptr(),
              mask_d.numel(), tab.data_ptr(), K, T, out.data_ptr(), int(basis), dv.stream_ptr())
    return _out(out, mask)


def zernike(mask, index, normalize=True, order='noll', rho=None, theta=None):
    """One Zernike polynomial over the nonzero pixels of ``mask``
    (lentil/zernike.py:11-93)."""
    return _eval(mask, [index], [1.0], normalize, order, rho, theta, basis=False)


def zernike_compose(mask, coeffs, normalize=True, order='noll', rho=None, theta=None):
    """sum_j coeffs[j-1] Z_j over ``mask`` (lentil/zernike.py:112-180)."""
    coeffs = np.asarray(coeffs, dtype=float).ravel()
    if coeffs.size == 0:
        z = torch.zeros(tuple(np.shape(mask)), dtype=torch.float64, device=dv.device())
        return _out(z, mask)
    return _eval(mask, range(1, coeffs.size + 1), coeffs, normalize, order, rho, theta,
                 basis=False)


def zernike_basis(mask, modes, vectorize=False, normalize=True, order='noll', rho=None,
                  theta=None):
    """Stack of Zernike polynomials, one per entry of ``modes``
    (lentil/zernike.py:183-234)."""
    modes = np.atleast_1d(np.asarray(modes)).ravel()
    basis = _eval(mask, [int(j) for j in modes], np.ones(modes.size), normalize, order, rho,
                  theta, basis=True)
    return basis.reshape(basis.shape[0], -1) if vectorize else basis
