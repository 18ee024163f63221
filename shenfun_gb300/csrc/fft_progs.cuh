// Block programs of the line transforms: tile staging, pre/post-processing of
// the Fourier and Chebyshev kinds, and the fused Shen-stencil / mass-solve
// epilogues.  Included at the end of fft_line.cuh.
//
// Element loops are two-dimensional (line x index along the line) with the
// thread decomposition computed once per loop, so no integer division runs
// per element.  Lines per CTA (tlc) are a power of two that divides the
// thread count; with a single emulated thread (the CPU harness) every loop
// degenerates to a full sequential sweep.
#pragma once

namespace sgpu {

// ---------------------------------------------------------------------------
// Tile addressing.  Lines are l = o * inner + i; a tile is TL consecutive
// lines.  Element (l, k) of an array with n_arr entries along the axis lives
// at o * n_arr * inner + k * inner + i.
SGPU_HD int64_t elem_off(int64_t l, int64_t k, int64_t n_arr, int64_t inner) {
  int64_t o = l / inner, i = l - o * inner;
  return (o * n_arr + k) * inner + i;
}

// Thread decomposition of an L x n loop: thread owns line c0 (+cstep ...) and
// indices k0, k0 + kstep, ...  When nth >= L every thread owns one line and
// the G = nth / L threads of a line stride along it; otherwise threads stride
// over lines and sweep each line fully.
struct LK {
  int c0, cstep, k0, kstep;
};

SGPU_HD LK lk_lines(int L, int tid, int nth) {
  LK m;
  if (nth >= L) {
    const int G = nth / L;
    m.c0 = tid / G;
    m.cstep = L;  // single pass; threads past G * L idle
    m.k0 = tid - m.c0 * G;
    m.kstep = G;
  } else {
    m.c0 = tid;
    m.cstep = nth;
    m.k0 = 0;
    m.kstep = 1;
  }
  return m;
}

// Transposed decomposition for strided tiles: consecutive threads take
// consecutive lines at the same k (row-coalesced loads when inner > 1).
SGPU_HD LK lk_rows(int L, int tid, int nth) {
  LK m;
  if (nth >= L) {
    m.c0 = tid % L;
    m.cstep = L;  // single pass over lines
    m.k0 = tid / L;
    m.kstep = nth / L;
    if (m.k0 >= m.kstep) m.k0 = 1 << 30;  // threads past kstep * L idle
  } else {
    m.c0 = tid;
    m.cstep = nth;
    m.k0 = 0;
    m.kstep = 1;
  }
  return m;
}

// Real data: slot t of a tile starting at real line l0 (= 2 x the tile's
// first complex slot) holds real line pair_line(...): complex slot C pairs
// lines 2j and 2j + 1 of block b (blocks of pb lines, pb = 0: one block), so
// pairs never cross a block.  With one block this is line l0 + t.
SGPU_HD int64_t pair_line(int64_t l0, int t, int64_t pb, int64_t nlines, bool& live) {
  const int64_t B = pb > 0 ? pb : nlines;
  const int64_t hp = (B + 1) / 2;
  const int64_t C = l0 / 2 + (t >> 1);
  const int64_t b = C / hp, j = C - b * hp;
  const int64_t i = 2 * j + (t & 1);
  live = i < B && b * B + i < nlines;
  return b * B + i;
}

// complex slots (pairs of real lines) of nlines real lines in blocks of pb
SGPU_HD int64_t pair_slots(int64_t nlines, int64_t pb) {
  const int64_t B = pb > 0 ? pb : nlines;
  if (B <= 0) return 0;
  const int64_t full = nlines / B, r = nlines - full * B;
  return full * ((B + 1) / 2) + (r + 1) / 2;
}

#define SGPU_FOR_LK(m, L, n, c, k)                  \
  for (int c = (m).c0; c < (L); c += (m).cstep)     \
    for (int k = (m).k0; k < (n); k += (m).kstep)

// Stencil coefficient K_m(k) of the Shen basis (offsets 0, 2, 4).  Constant
// entries (the 1 and -1 of ShenDirichlet, the leading 1 of ShenBiharmonic)
// apply to every row, as in the reference's stencil matrix
// (spectralbase.py:1504-1526); k-dependent entries are zero for k >= dim.
template <class R>
SGPU_HD R stencil_coef(const LinePlan& p, int off, int k) {
  if (p.basis == SGPU_BASIS_ORTHO) return off == 0 ? R(1.0) : R(0.0);
  if (p.basis == SGPU_BASIS_SD) return off == 0 ? R(1.0) : (off == 2 ? R(-1.0) : R(0.0));
  if (off == 0) return R(1.0);
  if (off == 2) return sten_at<R>(p, k);
  if (off == 4) return sten_at<R>(p, p.n + k);
  return R(0.0);
}

SGPU_HD int basis_nbcs(int basis) {
  return (basis == SGPU_BASIS_SD || basis == SGPU_BASIS_SN) ? 2 : (basis == SGPU_BASIS_SB ? 4 : 0);
}

// ---------------------------------------------------------------------------
// Shared memory: X | A | B (tlc * ld complex each) | slot (2 tlc).  A and B
// are contiguous, so 2 * tlc lines of stride ld fit in A..B.
template <class R>
struct Smem {
  Cx<R>* X;
  Cx<R>* A;
  Cx<R>* B;
  Cx<R>* slot;
};

template <class R>
SGPU_HD Smem<R> carve(const LinePlan& p, void* smem) {
  Smem<R> s;
  Cx<R>* base = (Cx<R>*)smem;
  size_t L = (size_t)p.tlc * p.ld;
  s.X = base;
  s.A = base + L;
  s.B = base + 2 * L;
  s.slot = base + 3 * L;
  return s;
}

template <class R>
SGPU_HD size_t smem_bytes(int tlc, int ld) {
  return sizeof(Cx<R>) * ((size_t)3 * tlc * ld + 2 * (size_t)tlc);
}

// Load TL lines into X.  Real data: line pair (2c, 2c+1) -> complex line c
// (re, im); complex data: line c -> complex line c.  Lines past the end of
// the array read as zero.
// paired: the tile's lines are the real-line pairs of its complex slots
// (R2C, C2R, real DCTs), placed by pair_line; otherwise line l0 + t.
template <class R>
SGPU_HD void load_tile(const LinePlan& p, const void* in, int in_complex, int paired, int TL, int n_arr,
                       int64_t l0, int64_t nlines, int64_t inner, Cx<R>* X, int tid, int nth) {
  if (inner == 1) {
    const LK m = lk_lines(TL, tid, nth);
    for (int t = m.c0; t < TL; t += m.cstep) {
      bool live = l0 + t < nlines;
      const int64_t l = paired ? pair_line(l0, t, p.pb, nlines, live) : l0 + t;
      if (in_complex) {
        const double* src = (const double*)in + 2 * (l * n_arr);
        Cx<R>* dst = X + (size_t)t * p.ld;
        for (int k = m.k0; k < n_arr; k += m.kstep)
          dst[k] = live ? cx<R>(from_f64<R>(src[2 * k]), from_f64<R>(src[2 * k + 1]))
                        : cx<R>(R(0.0), R(0.0));
      } else {
        const double* src = (const double*)in + l * n_arr;
        R* dst = (R*)(X + (size_t)(t >> 1) * p.ld) + (t & 1);
        for (int k = m.k0; k < n_arr; k += m.kstep) dst[2 * k] = live ? from_f64<R>(src[k]) : R(0.0);
      }
    }
  } else {
    const LK m = lk_rows(TL, tid, nth);
    for (int t = m.c0; t < TL; t += m.cstep) {
      bool live = l0 + t < nlines;
      const int64_t l = paired ? pair_line(l0, t, p.pb, nlines, live) : l0 + t;
      const int64_t base = live ? elem_off(l, 0, n_arr, inner) : 0;
      for (int k = m.k0; k < n_arr; k += m.kstep) {
        const int64_t off = base + (int64_t)k * inner;
        if (in_complex) {
          const double* src = (const double*)in + 2 * off;
          X[(size_t)t * p.ld + k] = live ? cx<R>(from_f64<R>(src[0]), from_f64<R>(src[1]))
                                         : cx<R>(R(0.0), R(0.0));
        } else {
          R* dst = (R*)(X + (size_t)(t >> 1) * p.ld) + (t & 1);
          dst[2 * k] = live ? from_f64<R>(((const double*)in)[off]) : R(0.0);
        }
      }
    }
  }
  SGPU_SYNC();
}

// Store TL lines from Y (complex lines, or real line pairs packed re/im).
template <class R>
SGPU_HD void store_tile(const LinePlan& p, void* out, int out_complex, int paired, int TL, int n_arr,
                        int64_t l0, int64_t nlines, int64_t inner, const Cx<R>* Y, int tid,
                        int nth) {
  if (inner == 1) {
    const LK m = lk_lines(TL, tid, nth);
    for (int t = m.c0; t < TL; t += m.cstep) {
      bool live = l0 + t < nlines;
      const int64_t l = paired ? pair_line(l0, t, p.pb, nlines, live) : l0 + t;
      if (!live) continue;
      if (out_complex) {
        double* dst = (double*)out + 2 * (l * n_arr);
        const Cx<R>* src = Y + (size_t)t * p.ld;
        for (int k = m.k0; k < n_arr; k += m.kstep) {
          const Cx<R> v = src[k];
          dst[2 * k] = to_f64(v.re);
          dst[2 * k + 1] = to_f64(v.im);
        }
      } else {
        double* dst = (double*)out + l * n_arr;
        const R* src = (const R*)(Y + (size_t)(t >> 1) * p.ld) + (t & 1);
        for (int k = m.k0; k < n_arr; k += m.kstep) dst[k] = to_f64(src[2 * k]);
      }
    }
  } else {
    const LK m = lk_rows(TL, tid, nth);
    for (int t = m.c0; t < TL; t += m.cstep) {
      bool live = l0 + t < nlines;
      const int64_t l = paired ? pair_line(l0, t, p.pb, nlines, live) : l0 + t;
      if (!live) continue;
      const int64_t base = elem_off(l, 0, n_arr, inner);
      for (int k = m.k0; k < n_arr; k += m.kstep) {
        const int64_t off = base + (int64_t)k * inner;
        if (out_complex) {
          const Cx<R> v = Y[(size_t)t * p.ld + k];
          double* dst = (double*)out + 2 * off;
          dst[0] = to_f64(v.re);
          dst[1] = to_f64(v.im);
        } else {
          const R* src = (const R*)(Y + (size_t)(t >> 1) * p.ld) + (t & 1);
          ((double*)out)[off] = to_f64(src[2 * k]);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Fourier R2C: pairs of real lines -> half spectra, times `scale`.
template <class R>
SGPU_HD void prog_r2c(const LinePlan& p, const double* in, double* out, int64_t nlines,
                      int64_t inner, double scl, int64_t blk, void* smem, int tid, int nth) {
  Smem<R> s = carve<R>(p, smem);
  const int64_t l0 = blk * 2 * p.tlc;
  load_tile<R>(p, in, 0, 1, 2 * p.tlc, p.n_in, l0, nlines, inner, s.X, tid, nth);
  dft_lines<R>(p, s.X, s.A, s.B, s.slot, p.tlc, tid, nth);
  // P_k = (Z_k + conj Z_{n-k}) / 2, Q_k = (Z_k - conj Z_{n-k}) / (2i)
  const int n = p.n, nh = n / 2 + 1;
  const R h = R(0.5) * from_f64<R>(scl);
  const LK m = lk_lines(p.tlc, tid, nth);
  SGPU_FOR_LK(m, p.tlc, nh, c, k) {
    Cx<R> z = s.X[(size_t)c * p.ld + k];
    Cx<R> zc = conj(s.X[(size_t)c * p.ld + (k == 0 ? 0 : n - k)]);
    s.A[(size_t)(2 * c) * p.ld + k] = scale(z + zc, h);
    s.A[(size_t)(2 * c + 1) * p.ld + k] = scale(mul_mi(z - zc), h);
  }
  SGPU_SYNC();
  store_tile<R>(p, out, 1, 1, 2 * p.tlc, p.n_out, l0, nlines, inner, s.A, tid, nth);
}

// Fourier C2R: pairs of half spectra -> real lines (unnormalised), times scale.
template <class R>
SGPU_HD void prog_c2r(const LinePlan& p, const double* in, double* out, int64_t nlines,
                      int64_t inner, double scl, int64_t blk, void* smem, int tid, int nth) {
  Smem<R> s = carve<R>(p, smem);
  const int64_t l0 = blk * 2 * p.tlc;
  load_tile<R>(p, in, 1, 1, 2 * p.tlc, p.n_in, l0, nlines, inner, s.A, tid, nth);
  const int n = p.n, nh = n / 2 + 1;
  // Z_k = P_k + i Q_k with Hermitian extension; DC and (even n) Nyquist real;
  // conjugated for the inverse: IDFT(Z) = conj(DFT(conj Z))
  const LK m = lk_lines(p.tlc, tid, nth);
  SGPU_FOR_LK(m, p.tlc, n, c, k) {
    const Cx<R>* P = s.A + (size_t)(2 * c) * p.ld;
    const Cx<R>* Q = s.A + (size_t)(2 * c + 1) * p.ld;
    Cx<R> pk, qk;
    if (k < nh) {
      pk = P[k];
      qk = Q[k];
      if (k == 0 || 2 * k == n) {
        pk.im = R(0.0);
        qk.im = R(0.0);
      }
    } else {
      pk = conj(P[n - k]);
      qk = conj(Q[n - k]);
    }
    s.X[(size_t)c * p.ld + k] = conj(pk + mul_pi(qk));
  }
  SGPU_SYNC();
  dft_lines<R>(p, s.X, s.A, s.B, s.slot, p.tlc, tid, nth);
  const R sc = from_f64<R>(scl);
  SGPU_FOR_LK(m, p.tlc, n, c, k) {
    Cx<R> z = s.X[(size_t)c * p.ld + k];
    s.X[(size_t)c * p.ld + k] = cx<R>(z.re * sc, -(z.im * sc));
  }
  SGPU_SYNC();
  store_tile<R>(p, out, 0, 1, 2 * p.tlc, p.n_out, l0, nlines, inner, s.X, tid, nth);
}

// Fourier C2C forward / backward (unnormalised), times scale.
template <class R>
SGPU_HD void prog_c2c(const LinePlan& p, const double* in, double* out, int64_t nlines,
                      int64_t inner, double scl, int64_t blk, void* smem, int tid, int nth) {
  Smem<R> s = carve<R>(p, smem);
  const int64_t l0 = blk * p.tlc;
  const bool bwd = p.kind == SGPU_XF_C2C_BWD;
  load_tile<R>(p, in, 1, 0, p.tlc, p.n_in, l0, nlines, inner, s.X, tid, nth);
  const int n = p.n;
  const LK m = lk_lines(p.tlc, tid, nth);
  if (bwd) {
    SGPU_FOR_LK(m, p.tlc, n, c, k) s.X[(size_t)c * p.ld + k] = conj(s.X[(size_t)c * p.ld + k]);
    SGPU_SYNC();
  }
  dft_lines<R>(p, s.X, s.A, s.B, s.slot, p.tlc, tid, nth);
  const R sc = from_f64<R>(scl);
  SGPU_FOR_LK(m, p.tlc, n, c, k) {
    Cx<R> z = s.X[(size_t)c * p.ld + k];
    s.X[(size_t)c * p.ld + k] = bwd ? cx<R>(z.re * sc, -(z.im * sc)) : scale(z, sc);
  }
  SGPU_SYNC();
  store_tile<R>(p, out, 1, 0, p.tlc, p.n_out, l0, nlines, inner, s.X, tid, nth);
}

// Chebyshev forward kinds: DCT-II (REDFT10) and the GC scalar product with the
// stencil epilogue (+ inverse mass for SGPU_XF_CHEB_FORWARD).
template <class R>
SGPU_HD void prog_dct2(const LinePlan& p, const double* in, double* out, int in_complex,
                       int64_t nlines, int64_t inner, double scl, int64_t blk, void* smem,
                       int tid, int nth) {
  Smem<R> s = carve<R>(p, smem);
  const int TL = in_complex ? p.tlc : 2 * p.tlc;
  const int64_t l0 = blk * TL;
  const int n = p.n, h = (n + 1) / 2;
  load_tile<R>(p, in, in_complex, !in_complex, TL, n, l0, nlines, inner, s.A, tid, nth);
  const LK m = lk_lines(p.tlc, tid, nth);
  // Makhoul reorder: v_j = x_{2j} (j < h), v_{n-1-j} = x_{2j+1}
  SGPU_FOR_LK(m, p.tlc, n, c, j) {
    int src = j < h ? 2 * j : 2 * (n - 1 - j) + 1;
    s.X[(size_t)c * p.ld + j] = s.A[(size_t)c * p.ld + src];
  }
  SGPU_SYNC();
  dft_lines<R>(p, s.X, s.A, s.B, s.slot, p.tlc, tid, nth);
  // Y_k = 2 Re(exp(-i pi k / 2n) V_k) for each of the two packed real lines.
  const R fac = (p.kind == SGPU_XF_DCT2) ? from_f64<R>(2.0 * scl)
                                         : from_f64<R>(3.14159265358979323846264338327950288 / n);
  SGPU_FOR_LK(m, p.tlc, n, c, k) {
    Cx<R> z = s.X[(size_t)c * p.ld + k];
    Cx<R> zc = conj(s.X[(size_t)c * p.ld + (k == 0 ? 0 : n - k)]);
    Cx<R> P = scale(z + zc, R(0.5));
    Cx<R> Q = scale(mul_mi(z - zc), R(0.5));
    Cx<R> w = post_at<R>(p, k);
    R yp = (w.re * P.re - w.im * P.im) * fac;
    R yq = (w.re * Q.re - w.im * Q.im) * fac;
    s.A[(size_t)c * p.ld + k] = cx<R>(yp, yq);
  }
  SGPU_SYNC();
  Cx<R>* Y = s.A;
  if (p.kind == SGPU_XF_CHEB_SCALAR || p.kind == SGPU_XF_CHEB_FORWARD) {
    // out_k = sum_m K_m(k) y_{k+m}
    SGPU_FOR_LK(m, p.tlc, n, c, k) {
      const Cx<R>* y = s.A + (size_t)c * p.ld;
      Cx<R> acc = y[k];
      if (p.basis == SGPU_BASIS_SD) {
        if (k + 2 < n) acc = acc - y[k + 2];
      } else if (p.basis == SGPU_BASIS_SB || p.basis == SGPU_BASIS_SN) {
        if (k + 2 < n) acc = acc + scale(y[k + 2], stencil_coef<R>(p, 2, k));
        if (p.basis == SGPU_BASIS_SB && k + 4 < n) acc = acc + scale(y[k + 4], stencil_coef<R>(p, 4, k));
      }
      s.B[(size_t)c * p.ld + k] = acc;
    }
    SGPU_SYNC();
    Y = s.B;
  }
  if (p.kind == SGPU_XF_CHEB_FORWARD) {
    // B^{-1} on the first dim entries (TDMA_inner_solve_ptr / PDMA_inner_solve_ptr,
    // la.pyx:496-532), boundary dofs zero (homogeneous BCs).  The plan's mass
    // table holds the LU'd bands with the diagonal row replaced by its
    // reciprocal, so the solve multiplies instead of dividing.
    const int nb = basis_nbcs(p.basis), dim = n - nb;
    for (int c = tid; c < p.tlc; c += nth) {
      Cx<R>* u = Y + (size_t)c * p.ld;
      if (nb == 2) {
        const double* ld_ = p.mass;
        const double* di = p.mass + dim;
        const double* ud = p.mass + 2 * dim + 2;
        for (int i = 2; i < dim; ++i) u[i] = u[i] - scale(u[i - 2], from_f64<R>(ld_[i - 2]));
        u[dim - 1] = scale(u[dim - 1], from_f64<R>(di[dim - 1]));
        u[dim - 2] = scale(u[dim - 2], from_f64<R>(di[dim - 2]));
        for (int i = dim - 3; i >= 0; --i)
          u[i] = scale(u[i] - scale(u[i + 2], from_f64<R>(ud[i])), from_f64<R>(di[i]));
      } else if (nb == 4) {
        const double* a = p.mass;
        const double* b = p.mass + dim;
        const double* di = p.mass + 2 * dim;
        const double* ee = p.mass + 3 * dim + 2;
        const double* f = p.mass + 4 * dim + 4;
        u[2] = u[2] - scale(u[0], from_f64<R>(b[0]));
        u[3] = u[3] - scale(u[1], from_f64<R>(b[1]));
        for (int k = 4; k < dim; ++k)
          u[k] = u[k] - (scale(u[k - 2], from_f64<R>(b[k - 2])) + scale(u[k - 4], from_f64<R>(a[k - 4])));
        u[dim - 1] = scale(u[dim - 1], from_f64<R>(di[dim - 1]));
        u[dim - 2] = scale(u[dim - 2], from_f64<R>(di[dim - 2]));
        u[dim - 3] = scale(u[dim - 3] - scale(u[dim - 1], from_f64<R>(ee[dim - 3])), from_f64<R>(di[dim - 3]));
        u[dim - 4] = scale(u[dim - 4] - scale(u[dim - 2], from_f64<R>(ee[dim - 4])), from_f64<R>(di[dim - 4]));
        for (int k = dim - 5; k >= 0; --k)
          u[k] = scale(u[k] - scale(u[k + 2], from_f64<R>(ee[k])) - scale(u[k + 4], from_f64<R>(f[k])),
                       from_f64<R>(di[k]));
      } else {
        // orthogonal basis: diagonal mass; the table holds 1 / (c_k pi / 2)
        for (int k = 0; k < n; ++k) u[k] = scale(u[k], from_f64<R>(p.mass[k]));
      }
      for (int k = dim; k < n; ++k) u[k] = cx<R>(R(0.0), R(0.0));
    }
    SGPU_SYNC();
  }
  store_tile<R>(p, out, in_complex, !in_complex, TL, n, l0, nlines, inner, Y, tid, nth);
}

// Chebyshev backward kinds: DCT-III (REDFT01) and the GC backward with the
// to_ortho prologue (0.5 * REDFT01 + c_0 / 2).
template <class R>
SGPU_HD void prog_dct3(const LinePlan& p, const double* in, double* out, int in_complex,
                       int64_t nlines, int64_t inner, double scl, int64_t blk, void* smem,
                       int tid, int nth) {
  Smem<R> s = carve<R>(p, smem);
  const int TL = in_complex ? p.tlc : 2 * p.tlc;
  const int64_t l0 = blk * TL;
  const int n = p.n;
  load_tile<R>(p, in, in_complex, !in_complex, TL, n, l0, nlines, inner, s.A, tid, nth);
  const LK m = lk_lines(p.tlc, tid, nth);
  Cx<R>* C = s.A;
  if (p.kind == SGPU_XF_CHEB_BACKWARD && p.basis != SGPU_BASIS_ORTHO) {
    // to_ortho: c_{k+m} += K_m(k) u_k for k < dim (spectralbase.py:1616-1634)
    const int dim = n - basis_nbcs(p.basis);
    SGPU_FOR_LK(m, p.tlc, n, c, k) {
      const Cx<R>* u = s.A + (size_t)c * p.ld;
      Cx<R> acc = cx<R>(R(0.0), R(0.0));
      if (k < dim) acc = u[k];
      if (p.basis == SGPU_BASIS_SD) {
        if (k - 2 >= 0 && k - 2 < dim) acc = acc - u[k - 2];
      } else {
        if (k - 2 >= 0 && k - 2 < dim) acc = acc + scale(u[k - 2], stencil_coef<R>(p, 2, k - 2));
        if (p.basis == SGPU_BASIS_SB && k - 4 >= 0 && k - 4 < dim)
          acc = acc + scale(u[k - 4], stencil_coef<R>(p, 4, k - 4));
      }
      if (p.bcfun) {
        // boundary functions of the dofs u_dim, u_dim+1 (BoundaryValues.
        // _add_to_orthogonal, tensorproductspace.py:2072-2089): SD
        // (T0 -+ T1)/2, SN T1/2 -+ T2/8 (the reference's bc stencils)
        const Cx<R> g0 = u[dim], g1 = u[dim + 1];
        const int kb = p.basis == SGPU_BASIS_SD ? 0 : 1;
        if (k == kb) acc = acc + (scale(g0, R(0.5)) + scale(g1, R(0.5)));
        if (k == kb + 1) {
          const R w = p.basis == SGPU_BASIS_SD ? R(0.5) : R(0.125);
          acc = acc + (scale(g1, w) - scale(g0, w));
        }
      }
      s.B[(size_t)c * p.ld + k] = acc;
    }
    SGPU_SYNC();
    C = s.B;
  }
  // W_k = f (c_k - i c_{n-k}) exp(i pi k / 2n), c_n = 0; for the GC backward
  // f = 1/2 and W_0 = c_0 (0.5 REDFT01 + c_0/2); for raw REDFT01 f = 1.
  // Two real lines p, q packed: Z = W_p + i W_q, conjugated for the IDFT.
  const bool gc = p.kind == SGPU_XF_CHEB_BACKWARD;
  const R f = gc ? R(0.5) : R(1.0);
  SGPU_FOR_LK(m, p.tlc, n, c, k) {
    const Cx<R>* cl = C + (size_t)c * p.ld;
    Cx<R> a = cl[k];
    Cx<R> z;
    if (k == 0) {
      z = a;  // W_0 = c_0 (both lines)
    } else {
      Cx<R> b = cl[n - k];
      Cx<R> wp = cx<R>(a.re, -b.re);
      Cx<R> wq = cx<R>(a.im, -b.im);
      Cx<R> tw = conj(post_at<R>(p, k));  // exp(+i pi k / 2n)
      wp = scale(wp * tw, f);
      wq = scale(wq * tw, f);
      z = wp + mul_pi(wq);
    }
    s.X[(size_t)c * p.ld + k] = conj(z);
  }
  SGPU_SYNC();
  dft_lines<R>(p, s.X, s.A, s.B, s.slot, p.tlc, tid, nth);
  // y_{2j} = w_j, y_{2j+1} = w_{n-1-j}; w = conj(result); line p = Re w, q = Im w
  const R sc = gc ? R(1.0) : from_f64<R>(scl);
  SGPU_FOR_LK(m, p.tlc, n, c, i) {
    int j = (i & 1) ? (n - 1 - (i >> 1)) : (i >> 1);
    Cx<R> z = conj(s.X[(size_t)c * p.ld + j]);
    s.A[(size_t)c * p.ld + i] = scale(z, sc);
  }
  SGPU_SYNC();
  store_tile<R>(p, out, in_complex, !in_complex, TL, n, l0, nlines, inner, s.A, tid, nth);
}

template <class R>
SGPU_HD void prog_dispatch(const LinePlan& p, const double* in, double* out, int data_complex,
                           int64_t nlines, int64_t inner, double scl, int64_t blk, void* smem,
                           int tid, int nth) {
  switch (p.kind) {
    case SGPU_XF_R2C: prog_r2c<R>(p, in, out, nlines, inner, scl, blk, smem, tid, nth); break;
    case SGPU_XF_C2R: prog_c2r<R>(p, in, out, nlines, inner, scl, blk, smem, tid, nth); break;
    case SGPU_XF_C2C_FWD:
    case SGPU_XF_C2C_BWD: prog_c2c<R>(p, in, out, nlines, inner, scl, blk, smem, tid, nth); break;
    case SGPU_XF_DCT2:
    case SGPU_XF_CHEB_SCALAR:
    case SGPU_XF_CHEB_FORWARD:
      prog_dct2<R>(p, in, out, data_complex, nlines, inner, scl, blk, smem, tid, nth);
      break;
    case SGPU_XF_DCT3:
    case SGPU_XF_CHEB_BACKWARD:
      prog_dct3<R>(p, in, out, data_complex, nlines, inner, scl, blk, smem, tid, nth);
      break;
    default: break;
  }
}

// whether the lines are complex: fixed by the Fourier kinds, chosen by the
// caller for the Chebyshev kinds
SGPU_HD int data_complex_for(const LinePlan& p, int data_kind) {
  if (p.kind == SGPU_XF_R2C) return 0;
  if (p.kind == SGPU_XF_C2R || p.kind == SGPU_XF_C2C_FWD || p.kind == SGPU_XF_C2C_BWD) return 1;
  return data_kind == SGPU_COMPLEX ? 1 : 0;
}

// number of lines one CTA handles for this plan and data kind
SGPU_HD int lines_per_block(const LinePlan& p, int data_complex) {
  switch (p.kind) {
    case SGPU_XF_R2C:
    case SGPU_XF_C2R: return 2 * p.tlc;
    case SGPU_XF_C2C_FWD:
    case SGPU_XF_C2C_BWD: return p.tlc;
    default: return data_complex ? p.tlc : 2 * p.tlc;
  }
}

}  // namespace sgpu
