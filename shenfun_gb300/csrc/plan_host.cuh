// Host-side construction of a LinePlan and its tables (twiddles, Rader
// permutations and kernel spectrum, DCT post-twiddles, Shen stencil rows and
// the LU'd mass bands).  Used by sgpu_plan_create (which uploads the tables)
// and by the CPU index-check harness (which keeps them in host memory).
#pragma once

#include <algorithm>
#include <thread>

#include <cmath>
#include <cstring>
#include <vector>

#include "ddouble.h"
#include "fft_line.cuh"

namespace sgpu {

struct HostTables {
  std::vector<cd> tw, rk, post;
  std::vector<int> rin, rout;
  std::vector<double> mass, sten;
  std::vector<Cx<df>> tw_f, rk_f, post_f;
  std::vector<df> sten_f;
  std::vector<int> tw_q;
};

// round(x 2^62) of a double-double |x| <= 1, split as h 2^31 + l with
// l in [0, 2^31) (+1, whose h does not fit, saturates)
inline void dd_to_q62(const ddm::dd& x, int* out) {
  const double two62 = 4611686018427387904.0;
  const double hv = x.hi * two62;  // exact: a power-of-two scaling
  long long q;
  if (hv >= two62) {
    q = (1LL << 62) - 1;
  } else {
    // hv is an integer when |x.hi| >= 2^-9 (53-bit significand scaled by
    // 2^62); the fraction and the low part add their rounded value
    const double hf = std::floor(hv);
    q = (long long)hf + (long long)std::llround((hv - hf) + x.lo * two62);
  }
  out[0] = (int)(q >> 31);
  out[1] = (int)(q & 0x7FFFFFFFLL);
}

// double-double -> double-float pair (hi = the float nearest to the FP64
// rounding, lo = the float nearest to the rest)
inline df dd_to_df(const ddm::dd& x) {
  const float h = (float)x.hi;
  const ddm::dd r = x - ddm::dd((double)h);
  return df(h, (float)(r.hi + r.lo));
}

namespace planhost {

using ddm::dd;

bool is_prime(int n) {
  if (n < 2) return false;
  for (int d = 2; d * d <= n; ++d)
    if (n % d == 0) return false;
  return true;
}

int powmod(long long b, long long e, long long m) {
  long long r = 1 % m;
  b %= m;
  while (e > 0) {
    if (e & 1) r = r * b % m;
    b = b * b % m;
    e >>= 1;
  }
  return (int)r;
}

int primitive_root(int p) {
  std::vector<int> qs;
  int phi = p - 1, x = phi;
  for (int d = 2; d * d <= x; ++d)
    if (x % d == 0) {
      qs.push_back(d);
      while (x % d == 0) x /= d;
    }
  if (x > 1) qs.push_back(x);
  for (int g = 2; g < p; ++g) {
    bool ok = true;
    for (int q : qs)
      if (powmod(g, phi / q, p) == 1) {
        ok = false;
        break;
      }
    if (ok) return g;
  }
  return -1;
}

// radix sequence for a length-m Stockham FFT: 4s first, then 2, 3, 5, then
// remaining primes through the generic radix.
bool factorize(int m, int* radix, int* ns) {
  int k = 0;
  while (m % 4 == 0) {
    radix[k++] = 4;
    m /= 4;
  }
  const int small[3] = {2, 3, 5};
  for (int r : small)
    while (m % r == 0) {
      radix[k++] = r;
      m /= r;
    }
  for (int p = 7; m > 1; p += 2) {
    while (m % p == 0) {
      if (p > SGPU_MAX_GENERIC_RADIX || k >= SGPU_MAX_STAGES) return false;
      radix[k++] = p;
      m /= p;
    }
  }
  *ns = k;
  return k <= SGPU_MAX_STAGES;
}

}  // namespace planhost


// Fill p (device pointers left null) and the host tables; returns a status.
inline int build_plan_host(int kind, int n, int basis, int form, LinePlan& p, HostTables& T) {
  using namespace planhost;
  if (n < 2 || n > (1 << 20)) return SGPU_ERR_ARG;
  if (kind < SGPU_XF_R2C || kind > SGPU_XF_CHEB_BACKWARD) return SGPU_ERR_ARG;
  if (form != SGPU_PLAIN_F64 && form != SGPU_MIXED_DF) return SGPU_ERR_UNSUPPORTED;
  const bool cheb = kind >= SGPU_XF_DCT2;
  const bool composite = kind >= SGPU_XF_CHEB_SCALAR;
  const int bcflag = basis & SGPU_BASIS_BC;
  basis &= ~SGPU_BASIS_BC;
  if (composite && (basis < SGPU_BASIS_ORTHO || basis > SGPU_BASIS_SN)) return SGPU_ERR_ARG;
  if (bcflag && !(composite && (basis == SGPU_BASIS_SD || basis == SGPU_BASIS_SN))) return SGPU_ERR_ARG;
  if (composite && n < 2 + 2 * basis_nbcs(basis)) return SGPU_ERR_ARG;
  std::memset(&p, 0, sizeof(p));
  p.form = form;
  p.kind = kind;
  p.basis = composite ? basis : SGPU_BASIS_ORTHO;
  p.bcfun = (bcflag && kind == SGPU_XF_CHEB_BACKWARD) ? 1 : 0;
  p.n = n;
  p.n_in = (kind == SGPU_XF_C2R) ? n / 2 + 1 : n;
  p.n_out = (kind == SGPU_XF_R2C) ? n / 2 + 1 : n;
  p.rader = (is_prime(n) && n >= 11) ? 1 : 0;
  p.m = p.rader ? n - 1 : n;
  if (!factorize(p.m, p.radix, &p.nstages)) return SGPU_ERR_UNSUPPORTED;
  // line stride: >= n and >= m + P for the two-pass exchange buffer of the
  // register FFT (P <= 16 for the lengths that have one)
  const bool fast = p.m == 16 || p.m == 32 || p.m == 64 || p.m == 128 || p.m == 256;
  p.ld = fast ? (n > p.m + 16 ? n : p.m + 16) : n;
  p.nthreads = 256;
  // lines per CTA: X, A, B line buffers within ~96 KB of shared memory
  const size_t per_line = 3 * sizeof(cd) * (size_t)p.ld + 2 * sizeof(cd);
  int tlc = (int)((96 * 1024) / per_line);
  if (tlc > 16) tlc = 16;
  if (tlc < 1) tlc = 1;
  // a power of two, so that the line loops split the 256 threads evenly
  while (tlc & (tlc - 1)) tlc &= tlc - 1;
  p.tlc = tlc;
  p.smem = smem_bytes<double>(p.tlc, p.ld);
  if (p.smem > 220 * 1024) return SGPU_ERR_UNSUPPORTED;

  // ---- host tables -------------------------------------------------------
  const int m = p.m;
  std::vector<cd>& tw = T.tw;
  std::vector<cd>& rk = T.rk;
  std::vector<cd>& post = T.post;
  std::vector<int>& rin = T.rin;
  std::vector<int>& rout = T.rout;
  std::vector<double>& mass = T.mass;
  std::vector<double>& sten = T.sten;
  tw.resize(m);
  T.tw_f.resize(m);
  if (m == 256) T.tw_q.resize(4 * (size_t)m);
  for (int e = 0; e < m; ++e) {
    dd c, s;  // exp(-2 pi i e / m)
    ddm::sincos_2pi_frac(-e, m, c, s);
    tw[e] = cx<double>(ddm::to_double(c), ddm::to_double(s));
    T.tw_f[e] = cx<df>(dd_to_df(c), dd_to_df(s));
    if (m == 256) {
      dd_to_q62(c, &T.tw_q[4 * (size_t)e]);
      dd_to_q62(s, &T.tw_q[4 * (size_t)e + 2]);
    }
  }
  if (p.rader) {
    const int g = primitive_root(n);
    const int ginv = powmod(g, n - 2, n);
    rin.resize(m);
    rout.resize(m);
    for (int q = 0; q < m; ++q) {
      rin[q] = powmod(g, q, n);
      rout[q] = powmod(ginv, q, n);
    }
    // rk = DFT_m(b) / m with b_q = exp(-2 pi i ginv^q / n)
    std::vector<dd> br(m), bi(m);
    for (int q = 0; q < m; ++q) ddm::sincos_2pi_frac(-(int64_t)rout[q], n, br[q], bi[q]);
    // m-th roots of unity once (double-double), indexed by q s mod m
    std::vector<dd> wr(m), wi(m);
    for (int e = 0; e < m; ++e) ddm::sincos_2pi_frac(-e, m, wr[e], wi[e]);
    rk.resize(m);
    T.rk_f.resize(m);
    // O(m^2) in double-double: the outputs s are independent, spread over
    // the host's cores
    auto rk_range = [&](int s0, int s1) {
      for (int s = s0; s < s1; ++s) {
        dd sr, si;
        int e = 0;  // q * s mod m
        for (int q = 0; q < m; ++q) {
          const dd& c = wr[e];
          const dd& sn = wi[e];
          sr += br[q] * c - bi[q] * sn;
          si += br[q] * sn + bi[q] * c;
          e += s;
          if (e >= m) e -= m;
        }
        const dd rr = sr / (double)m, ri = si / (double)m;
        rk[s] = cx<double>(ddm::to_double(rr), ddm::to_double(ri));
        T.rk_f[s] = cx<df>(dd_to_df(rr), dd_to_df(ri));
      }
    };
    const unsigned hw = std::thread::hardware_concurrency();
    const int nth = m >= 64 ? (int)std::min(hw ? hw : 1u, 16u) : 1;
    std::vector<std::thread> pool;
    for (int t = 1; t < nth; ++t) pool.emplace_back(rk_range, (int)((int64_t)m * t / nth), (int)((int64_t)m * (t + 1) / nth));
    rk_range(0, (int)((int64_t)m / nth));
    for (auto& th : pool) th.join();
  }
  if (cheb) {
    post.resize(n);
    for (int k = 0; k < n; ++k) {
      dd c, s;  // exp(-i pi k / (2 n)) = exp(-2 pi i k / (4 n))
      ddm::sincos_2pi_frac(-k, 4 * (int64_t)n, c, s);
      post[k] = cx<double>(ddm::to_double(c), ddm::to_double(s));
      T.post_f.push_back(cx<df>(dd_to_df(c), dd_to_df(s)));
    }
  }
  if (p.basis == SGPU_BASIS_SB) {
    // K2(k) = -(2k+4)/(k+3), K4(k) = (k+1)/(k+3), zero for k >= n-4
    sten.assign(2 * (size_t)n, 0.0);
    T.sten_f.assign(2 * (size_t)n, df());
    for (int k = 0; k < n - 4; ++k) {
      sten[k] = -(2.0 * k + 4) / (k + 3.0);
      sten[n + k] = (k + 1.0) / (k + 3.0);
      T.sten_f[k] = dd_to_df(-(dd(2.0 * k + 4) / (k + 3.0)));
      T.sten_f[n + k] = dd_to_df(dd(k + 1.0) / (k + 3.0));
    }
  }
  if (p.basis == SGPU_BASIS_SN) {
    // K2(k) = -(k/(k+2))^2 for k < n-2 (chebyshev/bases.py:937), no K4
    sten.assign(2 * (size_t)n, 0.0);
    T.sten_f.assign(2 * (size_t)n, df());
    for (int k = 0; k < n - 2; ++k) {
      const double r = k / (k + 2.0);
      const dd rl = dd((double)k) / (k + 2.0);
      sten[k] = -(r * r);
      T.sten_f[k] = dd_to_df(-(rl * rl));
    }
  }
  if (kind == SGPU_XF_CHEB_FORWARD) {
    // Chebyshev mass matrices (chebyshev/matrices.py:238-246, :515-528), LU'd
    // as la.pyx:213-252 do, diagonal row replaced by its reciprocal.
    const double pi = 3.14159265358979323846;
    std::vector<double> h(n, pi / 2);
    h[0] = pi;
    if (p.basis == SGPU_BASIS_ORTHO) {
      mass.resize(n);
      for (int k = 0; k < n; ++k) mass[k] = 1.0 / h[k];
    } else if (p.basis == SGPU_BASIS_SD || p.basis == SGPU_BASIS_SN) {
      // SN: BSNSN (chebyshev/matrices.py:377-401), b_kk = h_k + K2(k)^2 h_{k+2},
      // b_{k,k+2} = b_{k+2,k} = K2(k) h_{k+2}
      const int dim = n - 2;
      mass.assign(3 * (size_t)dim, 0.0);
      double* ldg = &mass[0];
      double* d = &mass[dim];
      double* ud = &mass[2 * dim + 2];
      if (p.basis == SGPU_BASIS_SD) {
        for (int k = 0; k < dim; ++k) d[k] = h[k] + h[k + 2];
        for (int k = 0; k < dim - 2; ++k) ldg[k] = ud[k] = -h[1];
      } else {
        for (int k = 0; k < dim; ++k) {
          const double al = (k / (k + 2.0)) * (k / (k + 2.0));
          d[k] = h[k] + al * al * h[k + 2];
        }
        for (int k = 0; k < dim - 2; ++k) {
          const double al = (k / (k + 2.0)) * (k / (k + 2.0));
          ldg[k] = ud[k] = -al * h[k + 2];
        }
      }
      for (int i = 2; i < dim; ++i) {
        ldg[i - 2] = ldg[i - 2] / d[i - 2];
        d[i] = d[i] - ldg[i - 2] * ud[i - 2];
      }
      for (int k = 0; k < dim; ++k) d[k] = 1.0 / d[k];
    } else {
      const int dim = n - 4;
      std::vector<double> K2(n, 0.0), K4(n, 0.0);
      for (int k = 0; k < n - 4; ++k) {
        K2[k] = -(2.0 * k + 4) / (k + 3.0);
        K4[k] = (k + 1.0) / (k + 3.0);
      }
      mass.assign(5 * (size_t)dim, 0.0);
      double* a = &mass[0];
      double* b = &mass[dim];
      double* d = &mass[2 * dim];
      double* e = &mass[3 * dim + 2];
      double* f = &mass[4 * dim + 4];
      for (int k = 0; k < dim; ++k) d[k] = h[k] + h[k + 2] * K2[k] * K2[k] + h[k + 4] * K4[k] * K4[k];
      for (int k = 0; k < dim - 2; ++k)
        b[k] = e[k] = h[k + 2] * K2[k] + h[k + 4] * K4[k] * K2[k + 2];
      for (int k = 0; k < dim - 4; ++k) a[k] = f[k] = h[k + 4] * K4[k];
      const int kk = 2;
      for (int i = 0; i < dim - 2 * kk; ++i) {
        double lam = b[i] / d[i];
        d[i + kk] -= lam * e[i];
        e[i + kk] -= lam * f[i];
        b[i] = lam;
        lam = a[i] / d[i];
        b[i + kk] -= lam * e[i];
        d[i + 2 * kk] -= lam * f[i];
        a[i] = lam;
      }
      for (int i = dim - 4; i <= dim - 3; ++i) {
        double lam = b[i] / d[i];
        d[i + kk] -= lam * e[i];
        b[i] = lam;
      }
      for (int k = 0; k < dim; ++k) d[k] = 1.0 / d[k];
    }
  }

  return SGPU_OK;
}

// Point a plan's table pointers into one contiguous table image at `base`
// (device or host); `off` receives the byte layout.  Returns total bytes.
#define SGPU_NTAB 12
inline size_t table_layout(const HostTables& T, size_t off[SGPU_NTAB]) {
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t sizes[SGPU_NTAB] = {
      sizeof(cd) * T.tw.size(),       sizeof(cd) * T.rk.size(),
      sizeof(int) * T.rin.size(),     sizeof(int) * T.rout.size(),
      sizeof(cd) * T.post.size(),     sizeof(double) * T.mass.size(),
      sizeof(double) * T.sten.size(), sizeof(Cx<df>) * T.tw_f.size(),
      sizeof(Cx<df>) * T.rk_f.size(), sizeof(Cx<df>) * T.post_f.size(),
      sizeof(df) * T.sten_f.size(),   sizeof(int) * T.tw_q.size()};
  size_t sz = 0;
  for (int i = 0; i < SGPU_NTAB; ++i) {
    off[i] = sz;
    sz += al(sizes[i]);
  }
  return sz;
}

inline void table_image(const HostTables& T, const size_t off[SGPU_NTAB], unsigned char* img) {
  auto cp = [&](int i, const void* src, size_t bytes) {
    if (bytes) std::memcpy(img + off[i], src, bytes);
  };
  cp(0, T.tw.data(), sizeof(cd) * T.tw.size());
  cp(1, T.rk.data(), sizeof(cd) * T.rk.size());
  cp(2, T.rin.data(), sizeof(int) * T.rin.size());
  cp(3, T.rout.data(), sizeof(int) * T.rout.size());
  cp(4, T.post.data(), sizeof(cd) * T.post.size());
  cp(5, T.mass.data(), sizeof(double) * T.mass.size());
  cp(6, T.sten.data(), sizeof(double) * T.sten.size());
  cp(7, T.tw_f.data(), sizeof(Cx<df>) * T.tw_f.size());
  cp(8, T.rk_f.data(), sizeof(Cx<df>) * T.rk_f.size());
  cp(9, T.post_f.data(), sizeof(Cx<df>) * T.post_f.size());
  cp(10, T.sten_f.data(), sizeof(df) * T.sten_f.size());
  cp(11, T.tw_q.data(), sizeof(int) * T.tw_q.size());
}

inline void bind_tables(LinePlan& p, const HostTables& T, const size_t off[SGPU_NTAB],
                        unsigned char* b) {
  p.tw = (const cd*)(b + off[0]);
  p.rk = T.rk.empty() ? nullptr : (const cd*)(b + off[1]);
  p.rin = T.rin.empty() ? nullptr : (const int*)(b + off[2]);
  p.rout = T.rout.empty() ? nullptr : (const int*)(b + off[3]);
  p.post = T.post.empty() ? nullptr : (const cd*)(b + off[4]);
  p.mass = T.mass.empty() ? nullptr : (const double*)(b + off[5]);
  p.sten = T.sten.empty() ? nullptr : (const double*)(b + off[6]);
  p.tw_f = (const Cx<df>*)(b + off[7]);
  p.rk_f = T.rk_f.empty() ? nullptr : (const Cx<df>*)(b + off[8]);
  p.post_f = T.post_f.empty() ? nullptr : (const Cx<df>*)(b + off[9]);
  p.sten_f = T.sten_f.empty() ? nullptr : (const df*)(b + off[10]);
  p.tw_q = T.tw_q.empty() ? nullptr : (const int*)(b + off[11]);
}

}  // namespace sgpu
