"""Padded (3/2-rule dealiased) transforms along Fourier axes (CPU oracle, numpy).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates FourierBase._padding_backward / _truncation_forward
(fourier/bases.py:409-435 for R2C, :570-598 for C2C) and the padded plans of
FourierBase.plan (:255-279): a backward transform zero-pads the N spectral
coefficients to M = floor(padding N) (an even N's Nyquist coefficient is
shared: halved, and for R2C made real) and runs the unnormalised inverse
transform of length M; a forward transform runs the length-M transform scaled
by 1/M and truncates back to N (an even N's Nyquist coefficient collects both
halves: summed for C2C, twice the real part for R2C).  Polynomial axes are
not padded here (padding factor 1).
"""
import numpy as np
import scipy.fft as sfft

from . import problems as P


def padded_length(N, factor):
    return int(np.floor(factor * N))


def _sl(ndim, axis, s):
    idx = [slice(None)] * ndim
    idx[axis] = s
    return tuple(idx)


def pad(u, kind, N, M, axis):
    """Spectral coefficients of length N (N//2+1 for R2C) -> padded ones."""
    shape = list(u.shape)
    nd = u.ndim
    if kind == "R2C":
        shape[axis] = M // 2 + 1
        out = np.zeros(shape, dtype=complex)
        out[_sl(nd, axis, slice(0, N // 2 + 1))] = u[_sl(nd, axis, slice(0, N // 2 + 1))]
        if N % 2 == 0:
            s = _sl(nd, axis, N // 2)
            out[s] = out[s].real * 0.5
        return out
    shape[axis] = M
    out = np.zeros(shape, dtype=complex)
    out[_sl(nd, axis, slice(0, N // 2 + 1))] = u[_sl(nd, axis, slice(0, N // 2 + 1))]
    out[_sl(nd, axis, slice(M - N // 2, M))] = u[_sl(nd, axis, slice(N - N // 2, N))]
    if N % 2 == 0:
        out[_sl(nd, axis, N // 2)] *= 0.5
        out[_sl(nd, axis, M - N // 2)] *= 0.5
    return out


def truncate(p, kind, N, M, axis):
    """Padded spectral coefficients -> length N (N//2+1 for R2C)."""
    nd = p.ndim
    shape = list(p.shape)
    if kind == "R2C":
        shape[axis] = N // 2 + 1
        t = np.array(p[_sl(nd, axis, slice(0, N // 2 + 1))], dtype=complex)
        if N % 2 == 0:
            s = _sl(nd, axis, N // 2)
            t[s] = t[s].real * 2
        return t
    shape[axis] = N
    t = np.zeros(shape, dtype=complex)
    t[_sl(nd, axis, slice(0, N // 2 + 1))] = p[_sl(nd, axis, slice(0, N // 2 + 1))]
    t[_sl(nd, axis, slice(N - N // 2, N))] += p[_sl(nd, axis, slice(M - N // 2, M))]
    return t


def padded_backward(u_hat, bases, factors):
    """BackwardTransform with padded Fourier axes (first axis last applied in
    the forward chain, so the backward chain runs axes in order)."""
    out = u_hat
    for ax, ((fam, kind, N), f) in enumerate(zip(bases, factors)):
        if fam == "fourier" and f != 1:
            M = padded_length(N, f)
            p = pad(out, kind, N, M, ax)
            out = (sfft.irfft(p, n=M, axis=ax, norm="forward") if kind == "R2C"
                   else sfft.ifft(p, axis=ax, norm="forward"))
        else:
            out = P._backward_1d(out, (fam, kind, N), ax)
    return out


def padded_forward(f, bases, factors, scalar=False):
    """ForwardTransform (or ScalarTransform) from the padded grid."""
    out = f
    for ax in reversed(range(len(bases))):
        fam, kind, N = bases[ax]
        fac = factors[ax]
        if fam == "fourier" and fac != 1:
            M = padded_length(N, fac)
            p = (sfft.rfft(out, axis=ax) if kind == "R2C" else sfft.fft(out, axis=ax)) / M
            out = truncate(p, kind, N, M, ax)
        else:
            out = (P._scalar_1d if scalar else P._forward_1d)(out, (fam, kind, N), ax)
    return out
