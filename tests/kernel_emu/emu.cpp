// CPU harness for the kernels' block programs (test infrastructure).
//
// Runs the exact __host__ __device__ block programs of the CUDA library with
// one emulated thread per block, on exactly-sized heap buffers, so that a
// build with -fsanitize=address,undefined reports any index that leaves its
// buffer.  Shared memory is poisoned with NaN to expose reads of unwritten
// staging data.  Driven by tests/test_kernel_emu.py through binary files.
//
//   emu xform  kind n basis outer inner data_kind scale in.bin out.bin
//   emu hlu    N outer inner alfa.bin beta.bin out.bin        (d0|d1|d2|L)
//   emu hsolve N outer inner data_kind b.bin fac.bin out.bin   (fac = d0|d1|d2|L)
//   emu hmatvec N outer inner data_kind v.bin alfa.bin beta.bin out.bin
//   emu nlu|nsolve|ncached ...   the same with the Neumann branch (ShenNeumann)
//   emu nmatvec N outer inner data_kind v.bin alfa.bin beta.bin out.bin
//   emu padd|pann N outer inner data_kind scale b.bin out.bin   (Poisson ADD / ANN)
//   emu tdma|pdma n outer inner data_kind raw.bin u.bin out.bin (LU then solve)
//   emu ozaki  N nlines inner cplx precise in.bin M.bin out.bin (split-BF16 contraction)
//   emu ozakic N nlines inner cplx precise kchunk in.bin M.bin out.bin  (K blocks per launch)
//   emu lcf    N nlines cplx bn in.bin M.bin out.bin   (fused contraction, 64- or 32-line tiles)
//   emu tables kind n basis out.bin   (plan tables: tw, rk, post as FP64 pairs, then the
//                                      double-float tw_f, rk_f, post_f as (hi, lo) per part)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../../shenfun_gb300/csrc/plan_host.cuh"
#include "../../shenfun_gb300/csrc/solvers.cuh"
#include "../../shenfun_gb300/csrc/ozaki.cuh"
#include "../../shenfun_gb300/csrc/lc_fused.cuh"
#include "../../shenfun_gb300/csrc/ref_progs.cuh"
#include "../../shenfun_gb300/csrc/fft256.cuh"
#include "../../shenfun_gb300/csrc/fft256_fx.cuh"

using namespace sgpu;

static double* read_exact(const char* path, size_t count) {
  FILE* f = fopen(path, "rb");
  if (!f) {
    fprintf(stderr, "cannot open %s\n", path);
    exit(2);
  }
  double* buf = (double*)malloc(sizeof(double) * (count ? count : 1));
  size_t got = fread(buf, sizeof(double), count, f);
  fclose(f);
  if (got != count) {
    fprintf(stderr, "%s: expected %zu doubles, got %zu\n", path, count, got);
    exit(2);
  }
  return buf;
}

static void write_exact(const char* path, const double* buf, size_t count) {
  FILE* f = fopen(path, "wb");
  fwrite(buf, sizeof(double), count, f);
  fclose(f);
}

static int xform(int argc, char** argv) {
  if (argc < 11) return 2;
  int kind = atoi(argv[2]), n = atoi(argv[3]), basis = atoi(argv[4]);
  long long outer = atoll(argv[5]), inner = atoll(argv[6]);
  int data_kind = atoi(argv[7]);
  double scl = atof(argv[8]);
  const int form = getenv("SGPU_EMU_FORM") ? atoi(getenv("SGPU_EMU_FORM")) : SGPU_PLAIN_F64;
  LinePlan p;
  HostTables T;
  int st = build_plan_host(kind, n, basis, form, p, T);
  if (st != SGPU_OK) {
    fprintf(stderr, "plan status %d\n", st);
    return 3;
  }
  size_t off[SGPU_NTAB];
  size_t sz = table_layout(T, off);
  unsigned char* img = (unsigned char*)malloc(sz);
  table_image(T, off, img);
  bind_tables(p, T, off, img);
  const int dc = data_complex_for(p, data_kind);
  int in_c = dc, out_c = dc;
  if (kind == SGPU_XF_R2C) {
    in_c = 0;
    out_c = 1;
  }
  if (kind == SGPU_XF_C2R) {
    in_c = 1;
    out_c = 0;
  }
  const size_t nin = (size_t)outer * p.n_in * inner * (in_c ? 2 : 1);
  const size_t nout = (size_t)outer * p.n_out * inner * (out_c ? 2 : 1);
  double* in = read_exact(argv[9], nin);
  double* out = (double*)malloc(sizeof(double) * (nout ? nout : 1));
  for (size_t i = 0; i < nout; ++i) out[i] = std::numeric_limits<double>::quiet_NaN();
  const long long nlines = outer * inner;
  p.pb = getenv("SGPU_EMU_PB") ? atoll(getenv("SGPU_EMU_PB")) : 0;
  if (getenv("SGPU_EMU_TLC")) {  // lines per CTA below the plan's (small launches)
    const int t = atoi(getenv("SGPU_EMU_TLC"));
    if (t >= 1 && t <= p.tlc && (t & (t - 1)) == 0) {
      p.tlc = t;
      p.smem = smem_bytes<double>(p.tlc, p.ld);
    }
  }
  const int lpb = lines_per_block(p, dc);
  const long long nblocks = dc ? (nlines + lpb - 1) / lpb : (pair_slots(nlines, p.pb) + p.tlc - 1) / p.tlc;
  const size_t nsm = p.smem / sizeof(double);
  for (long long b = 0; b < nblocks; ++b) {
    double* smem = (double*)malloc(p.smem);
    for (size_t i = 0; i < nsm; ++i) smem[i] = std::numeric_limits<double>::quiet_NaN();
    if (form == SGPU_MIXED_DF)
      prog_dispatch<df>(p, in, out, dc, nlines, inner, scl, b, smem, 0, 1);
    else
      prog_dispatch<double>(p, in, out, dc, nlines, inner, scl, b, smem, 0, 1);
    free(smem);
  }
  write_exact(argv[10], out, nout);
  free(in);
  free(out);
  free(img);
  return 0;
}

// Strided length-256 Fourier passes (fft256.cuh): every thread of a CTA runs
// each phase in turn, with the CTA's barriers between the phases.
template <class R>
static void f256_block(int kind, const LinePlan& p, const f256::Args& a, int64_t blk, Cx<R>* Z) {
  using namespace f256;
  for (int t = 0; t < NT; ++t) {
    switch (kind) {
      case C2C_FWD: pass1<R, C2C_FWD>(p, a, blk, Z, t); break;
      case C2C_BWD: pass1<R, C2C_BWD>(p, a, blk, Z, t); break;
      case R2C: pass1<R, R2C>(p, a, blk, Z, t); break;
      default: pass1<R, C2R>(p, a, blk, Z, t); break;
    }
  }
  static Cx<R> v[NT][16];
  for (int t = 0; t < NT; ++t) pass2_dft<R>(Z, t, v[t]);
  if (kind == R2C) {
    for (int t = 0; t < NT; ++t) r2c_stash<R>(Z, t, v[t]);
    for (int t = 0; t < NT; ++t) r2c_post<R>(a, blk, Z, t, NT);
    return;
  }
  for (int t = 0; t < NT; ++t) {
    switch (kind) {
      case C2C_FWD: pass2_store<R, C2C_FWD>(a, blk, t, v[t]); break;
      case C2C_BWD: pass2_store<R, C2C_BWD>(a, blk, t, v[t]); break;
      default: pass2_store<R, C2R>(a, blk, t, v[t]); break;
    }
  }
}

// the fixed-point form of the same passes (fft256_fx.cuh)
template <int KIND>
static void f256_block_fx(const LinePlan& p, const f256::Args& a, int64_t blk, unsigned char* smem,
                          const f256::FxScale& s) {
  using namespace f256;
  if (KIND == C2C_FWD || KIND == C2C_BWD) {
    const FxShared sh = fx_shared(smem);
    static Cq v[NT][16];
    if (getenv("SGPU_EMU_TILE") && atoi(getenv("SGPU_EMU_TILE")) == 1) {
      // the tensor-copy kernel: the block's box {2 TL doubles, 256 rows} at
      // (2 (l0 mod inner), 0, l0 / inner) of the map {2 inner, 256, outer}
      // lands row-major in the exchange buffer (zeros past the extent), the
      // threads read their values there, then pass 1 runs on the registers
      const int64_t l0 = blk * TL, outer = a.nlines / a.inner;
      if (outer * a.inner != a.nlines || (outer > 1 && a.inner % TL != 0)) abort();
      const int64_t o = l0 / a.inner, i0 = l0 % a.inner;
      double* tile = (double*)sh.Z;
      for (int n = 0; n < N; ++n)
        for (int j = 0; j < 2 * TL; ++j) {
          const int64_t xj = 2 * i0 + j;
          tile[n * 2 * TL + j] = xj < 2 * a.inner ? a.in[(o * N + n) * 2 * a.inner + xj] : 0.0;
        }
      static double x[NT][32];
      static int et[NT];
      for (int t = 0; t < NT; ++t) et[t] = fx_c2c_load_tile(a, blk, sh, tile, t, x[t]);
      for (int t = 0; t < NT; ++t) fx_c2c_pass1_regs<KIND>(p, sh, t, x[t], et[t]);
    } else {
      for (int t = 0; t < NT; ++t) fx_c2c_pass1<KIND>(p, a, blk, sh, t);
    }
    for (int t = 0; t < NT; ++t) {
      const int E = fx_c2c_pass2(sh, t, v[t]);
      fx_c2c_store<KIND>(a, t, v[t], E, sh, s);
    }
    return;
  }
  const FxHalf sh = fxh_shared(smem);
  for (int t = 0; t < NT; ++t) {
    if (KIND == R2C)
      fxh_r2c_pass1(p, a, blk, sh, t);
    else
      fxh_c2r_pass1(p, a, blk, sh, t);
  }
  static Cq v[2 * NT][8];
  static int E[2 * NT];
  for (int i = 0; i < 2 * NT; ++i) E[i] = fxh_pass2(sh, i & 31, i >> 5, v[i]);
  if (KIND == R2C) {
    for (int i = 0; i < 2 * NT; ++i) fxh_r2c_stash(sh, i & 31, i >> 5, v[i], E[i]);
    for (int t = 0; t < NT; ++t) fxh_r2c_post(p, a, sh, t, NT, s);
    return;
  }
  for (int i = 0; i < 2 * NT; ++i) fxh_c2r_store(a, sh, i & 31, i >> 5, v[i], E[i], s);
}

static int f256_mode(int argc, char** argv) {
  // f256 kind outer inner scl in out   (kind: SGPU_XF_*; form from SGPU_EMU_FORM)
  if (argc < 8) return 2;
  const int xk = atoi(argv[2]);
  long long outer = atoll(argv[3]), inner = atoll(argv[4]);
  double scl = atof(argv[5]);
  const int form = getenv("SGPU_EMU_FORM") ? atoi(getenv("SGPU_EMU_FORM")) : SGPU_PLAIN_F64;
  LinePlan p;
  HostTables T;
  if (build_plan_host(xk, 256, 0, form, p, T) != SGPU_OK) return 3;
  size_t off[SGPU_NTAB];
  unsigned char* img = (unsigned char*)malloc(table_layout(T, off));
  table_image(T, off, img);
  bind_tables(p, T, off, img);
  int kind = xk == SGPU_XF_C2C_FWD ? f256::C2C_FWD : xk == SGPU_XF_C2C_BWD ? f256::C2C_BWD
             : xk == SGPU_XF_R2C ? f256::R2C : f256::C2R;
  const int in_c = kind != f256::R2C, out_c = kind != f256::C2R;
  const size_t nin = (size_t)outer * p.n_in * inner * (in_c ? 2 : 1);
  const size_t nout = (size_t)outer * p.n_out * inner * (out_c ? 2 : 1);
  double* in = read_exact(argv[6], nin);
  double* out = (double*)malloc(sizeof(double) * nout);
  for (size_t i = 0; i < nout; ++i) out[i] = std::numeric_limits<double>::quiet_NaN();
  const int64_t pbl = getenv("SGPU_EMU_PB") ? atoll(getenv("SGPU_EMU_PB")) : 0;
  f256::Args a{in, out, outer * inner, inner, scl, pbl};
  const int64_t nt = (getenv("SGPU_EMU_FX") && atoi(getenv("SGPU_EMU_FX")) && form == SGPU_MIXED_DF)
                        ? f256::fx_tiles(kind, a.nlines)
                        : f256::tiles(kind, a.nlines, pbl);
  const bool fx = getenv("SGPU_EMU_FX") && atoi(getenv("SGPU_EMU_FX")) && form == SGPU_MIXED_DF;
  const size_t zb = fx ? (kind == f256::R2C || kind == f256::C2R ? f256::fxh_smem_bytes() : f256::fx_smem_bytes())
                       : (form == SGPU_MIXED_DF ? f256::smem_bytes<df>() : f256::smem_bytes<double>());
  void* Z = malloc(zb);
  const f256::FxScale fs = f256::fx_scale(scl);
  for (int64_t b = 0; b < nt; ++b) {
    memset(Z, 0xff, zb);  // NaN patterns: unwritten entries show
    if (fx) {
      unsigned char* sm = (unsigned char*)Z;
      switch (kind) {
        case f256::C2C_FWD: f256_block_fx<f256::C2C_FWD>(p, a, b, sm, fs); break;
        case f256::C2C_BWD: f256_block_fx<f256::C2C_BWD>(p, a, b, sm, fs); break;
        case f256::R2C: f256_block_fx<f256::R2C>(p, a, b, sm, fs); break;
        default: f256_block_fx<f256::C2R>(p, a, b, sm, fs); break;
      }
    } else if (form == SGPU_MIXED_DF)
      f256_block<df>(kind, p, a, b, (Cx<df>*)Z);
    else
      f256_block<double>(kind, p, a, b, (Cx<double>*)Z);
  }
  write_exact(argv[7], out, nout);
  free(Z);
  free(in);
  free(out);
  free(img);
  return 0;
}

// Split-BF16 tensor-core contraction: the row-exponent, split and epilogue
// block functions run as in the kernels; the bulk copies are memcpy's with
// the kernel's offsets into an exactly-sized stand-in for shared memory, and
// each tcgen05.mma is modelled from its descriptors (operand element (m, k)
// at start + (k/8) LBO + (m/8) SBO + 16 (m%8) + 2 (k%8)) with the FP32
// accumulator rounded once per instruction.
template <class C>
static int ozaki_run(const oz::Geom& g, const double* in, const double* M, double* out) {
  using namespace oz;
  const int S = C::S, NACC = C::NACC, BN = C::BN, B_BYTES = C::B_BYTES, LBO_B = C::LBO_B;
  std::vector<int> eA((size_t)g.mtiles * BM);
  for (int64_t row = 0; row < (int64_t)g.mtiles * BM; ++row)
    eA[row] = exp_from_field(rowexp_partial(in, g, row, 0, 1));
  const size_t at_elems = (size_t)S * g.mtiles * g.nkb * A_ELEMS;
  uint16_t* At = (uint16_t*)malloc(at_elems * 2);
  for (size_t i = 0; i < at_elems; ++i) At[i] = 0x7FC0;  // BF16 NaN: unwritten shows
  {
    void* ssm = malloc((size_t)S * A_BYTES);
    for (int mt = 0; mt < g.mtiles; ++mt)
      for (int kb = 0; kb < g.nkb; ++kb) {
        for (size_t i = 0; i < (size_t)S * A_ELEMS; ++i) ((uint16_t*)ssm)[i] = 0x7FC0;  // BF16 NaN
        split_block<C::S>(in, eA.data(), At, g, mt, kb, ssm, 0, 1);
      }
    free(ssm);
  }
  const size_t bt_elems = matrix_tile_elems<C>(g.N);
  uint16_t* Bt = (uint16_t*)malloc(bt_elems * 2);
  int* eB = (int*)malloc(sizeof(int) * (size_t)g.ntiles * BN);
  split_matrix_host<C>(M, g.N, Bt, eB);
  const size_t AH = A_BYTES / 2, BH = B_BYTES / 2;
  const size_t stage_bytes = (size_t)S * (AH + BH);
  uint8_t* smem = (uint8_t*)malloc(STAGES * stage_bytes);
  std::vector<float> acc((size_t)NACC * BM * BN);
  const uint32_t idesc = tc::idesc_bf16_f32(BM, BN);
  if (((idesc >> 17) & 63) * 8 != BN || ((idesc >> 24) & 31) * 16 != BM) return 5;
  auto bf = [](const uint8_t* p) {
    uint16_t h;
    memcpy(&h, p, 2);
    uint32_t u = (uint32_t)h << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
  };
  // ATMEM: TMEM buffers of the A slices, [buffer][slice][lane 128][16 elements]
  std::vector<float> tA(C::ATMEM ? (size_t)2 * S * BM * 16 : 0, std::numeric_limits<float>::quiet_NaN());
  int64_t qg = 0;  // the MMA thread's step counter (selects the A buffer)
  for (int c = 0; c < num_chunks(g); ++c)
  for (int mt = 0; mt < g.mtiles; ++mt)
    for (int nt = 0; nt < g.ntiles; ++nt) {
      const Geom h = chunk_geom(g, c);  // one GEMM launch per K chunk
      uint32_t inited = 0;
      for (int ks = 0; ks < oz_steps(h); ++ks, ++qg) {
        const int st = ks % STAGES, kb = h.kb0 + (ks >> 1), hf = ks & 1;
        uint8_t* sbase = smem + st * stage_bytes;
        for (int s = 0; s < S; ++s) {
          memcpy(sbase + (size_t)s * AH,
                 At + (((int64_t)s * g.mtiles + mt) * g.nkb + kb) * A_ELEMS + hf * (A_ELEMS / 2), AH);
          memcpy(sbase + (size_t)S * AH + (size_t)s * BH,
                 Bt + (((int64_t)s * g.ntiles + nt) * g.nkb_b + kb) * C::B_ELEMS + hf * (C::B_ELEMS / 2), BH);
        }
        const int buf = (int)(qg & 1);
        if (C::ATMEM) {
          // tcgen05.cp 128x256b of each slice from its descriptor: row m -> lane m
          for (int s = 0; s < S; ++s) {
            const uint64_t ad = tc::sdesc_interleave((uint32_t)(st * stage_bytes + s * AH), LBO_A, SBO);
            auto field = [](uint64_t d, int sh) { return (uint32_t)(((d >> sh) & 0x3FFF) << 4); };
            const uint32_t as = field(ad, 0), al = field(ad, 16), asb = field(ad, 32);
            for (int m = 0; m < BM; ++m)
              for (int k = 0; k < 16; ++k) {
                const uint32_t pa = as + (k >> 3) * al + (m >> 3) * asb + (m & 7) * 16 + (k & 7) * 2;
                if (pa + 2 > STAGES * stage_bytes) return 6;
                tA[(((size_t)buf * S + s) * BM + m) * 16 + k] = bf(smem + pa);
              }
          }
        }
        for (int s = 0; s < S; ++s)
          for (int t = 0; t + s < S; ++t) {
            const uint32_t a_off = (uint32_t)(st * stage_bytes + s * AH);
            const uint32_t b_off = (uint32_t)(st * stage_bytes + S * AH + t * BH);
            const uint64_t ad = tc::sdesc_interleave(a_off, LBO_A, SBO);
            const uint64_t bd = tc::sdesc_interleave(b_off, LBO_B, SBO);
            auto field = [](uint64_t d, int sh) { return (uint32_t)(((d >> sh) & 0x3FFF) << 4); };
            const uint32_t as = field(ad, 0), al = field(ad, 16), asb = field(ad, 32);
            const uint32_t bs = field(bd, 0), bl = field(bd, 16), bsb = field(bd, 32);
            const int a = s + t < NACC - 1 ? s + t : NACC - 1;
            for (int m = 0; m < BM; ++m)
              for (int n = 0; n < BN; ++n) {
                double sum = 0;
                for (int k = 0; k < 16; ++k) {
                  const uint32_t pa = as + (k >> 3) * al + (m >> 3) * asb + (m & 7) * 16 + (k & 7) * 2;
                  const uint32_t pb = bs + (k >> 3) * bl + (n >> 3) * bsb + (n & 7) * 16 + (k & 7) * 2;
                  if (pa + 2 > STAGES * stage_bytes || pb + 2 > STAGES * stage_bytes) return 6;
                  const float av = C::ATMEM ? tA[(((size_t)buf * S + s) * BM + m) * 16 + k] : bf(smem + pa);
                  sum += (double)av * (double)bf(smem + pb);
                }
                float& d = acc[((size_t)a * BM + m) * BN + n];
                d = (float)(((inited >> a) & 1 ? (double)d : 0.0) + sum);
              }
            inited |= 1u << a;
          }
      }
      for (int m = 0; m < BM; ++m) {
        const int64_t row = (int64_t)mt * BM + m;
        if (row >= g.nrows) continue;
        for (int n = 0; n < BN; ++n) {
          const int col = nt * BN + n;
          if (col >= g.N) continue;
          uint32_t gb[C::NACC];
          for (int a = 0; a < NACC; ++a) memcpy(&gb[a], &acc[((size_t)a * BM + m) * BN + n], 4);
          const double v = combine_groups<C::NACC>(gb, eA[row] - 2 * W + eB[col]);
          double& o = out[row_offset(g, row, col)];
          o = h.accum ? o + v : v;
        }
      }
    }
  free(At);
  free(Bt);
  free(eB);
  free(smem);
  return 0;
}

// emu ozaki N nlines inner cplx precise in.bin M.bin out.bin
static int ozaki(int argc, char** argv) {
  // "ozakic" takes the K blocks per GEMM launch before the files
  const int chunked = std::string(argv[1]) == "ozakic";
  if (argc < 10 + chunked) return 2;
  const int N = atoi(argv[2]);
  const long long nlines = atoll(argv[3]), inner = atoll(argv[4]);
  const int cplx = atoi(argv[5]), precise = atoi(argv[6]);
  const size_t cnt = (size_t)nlines * N * (1 + cplx);
  argv += chunked;
  double* in = read_exact(argv[7], cnt);
  double* M = read_exact(argv[8], (size_t)N * N);
  int K = 0;  // as the library: 1 + the last nonzero row of M
  for (int k = 0; k < N; ++k)
    for (int n = 0; n < N; ++n)
      if (M[(size_t)k * N + n] != 0.0) K = k + 1;
  // precise: 0 CfgStd, 1 CfgPrec, 2 CfgPrecTmemA (A slices through TMEM)
  const int bn = precise == 2 ? oz::CfgPrecTmemA::BN : (precise ? oz::CfgPrec::BN : oz::CfgStd::BN);
  oz::Geom g = oz::make_geom(N, nlines, inner, cplx, bn, K);
  if (chunked) g.kchunk = atoi(argv[6]);  // argv shifted by one: the chunk argument
  double* out = (double*)malloc(sizeof(double) * cnt);
  for (size_t i = 0; i < cnt; ++i) out[i] = std::numeric_limits<double>::quiet_NaN();
  const int rc = precise == 2 ? ozaki_run<oz::CfgPrecTmemA>(g, in, M, out)
                 : precise   ? ozaki_run<oz::CfgPrec>(g, in, M, out)
                             : ozaki_run<oz::CfgStd>(g, in, M, out);
  if (rc) return rc;
  write_exact(argv[9], out, cnt);
  free(in);
  free(M);
  free(out);
  return 0;
}

// Fused split-BF16 contraction (lc_fused.cu): per tile, pass 1 (scales and
// FP64 dot-product outputs) over every cluster rank's share of rows, pass 2
// into a NaN-poisoned, exactly-sized B stage at the kernel's offsets for
// every K step, the MMAs of every rank modelled from their descriptors and
// instruction descriptors (operand element (m, k) at start + (k/8) LBO +
// (m/8) SBO + 16 (m%8) + 2 (k%8), FP32 accumulator rounded once per MMA), and
// the integer epilogue.
template <class C>
static int lcf_run(const lc::Geom& g, const double* in, const double* M, double* out) {
  using namespace lc;
  const int S = C::S, BN = C::BN;
  std::vector<uint16_t> tiles(matrix_tile_elems<C>(g));
  std::vector<int> em((size_t)g.MT * MROWS);
  std::vector<double> xcol((size_t)(g.NX > 0 ? g.NX : 1) * g.K);
  split_matrix_host<C>(M, g, tiles.data(), em.data(), xcol.data());
  std::vector<uint8_t> bst(C::B_STAGE), ast(C::A_STAGE);
  std::vector<int> e(BN);
  std::vector<double> xo((size_t)BN * MAX_NX);
  std::vector<float> D((size_t)g.MT * MROWS * S * BN);
  auto bf = [](const uint8_t* p) {
    uint16_t h;
    memcpy(&h, p, 2);
    uint32_t u = (uint32_t)h << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
  };
  auto field = [](uint64_t d, int sh) { return (uint32_t)(((d >> sh) & 0x3FFF) << 4); };
  const int ksd = kstride(g);
  for (int64_t T = 0; T < g.tiles; ++T) {
    const int64_t row0 = T * BN;
    for (int jj = 0; jj < BN; ++jj) {
      const int64_t row = row0 + jj;
      uint32_t mf = 0;
      double acc[MAX_NX] = {0.0, 0.0};
      if (row < g.nrows)
        for (int k = 0; k < g.K; ++k) {
          const double x = in[row_base(g, row) + (int64_t)k * ksd];
          mf = exp_field(x) > mf ? exp_field(x) : mf;
          for (int c = 0; c < g.NX; ++c) acc[c] += x * xcol[(size_t)c * g.K + k];
        }
      e[jj] = exp_from_field(mf);
      for (int c = 0; c < MAX_NX; ++c) xo[(size_t)jj * MAX_NX + c] = acc[c];
    }
    for (int ks = 0; ks < g.nsteps; ++ks) {
      for (size_t i = 0; i < bst.size(); i += 2) {
        bst[i] = 0xC0;
        bst[i + 1] = 0x7F;  // BF16 NaN: unwritten shows
      }
      {
        for (int h = 0; h < 2; ++h)
          for (int jj = 0; jj < BN; ++jj) {
            const int64_t row = row0 + jj;
            double x[8];
            const int k0 = ks * KSTEP + h * 8;
            for (int q = 0; q < 8; ++q)
              x[q] = row < g.nrows && k0 + q < g.K ? in[row_base(g, row) + (int64_t)(k0 + q) * ksd] : 0.0;
            uint4 dg[C::S];
            split8<C>(x, e[jj], dg);
            for (int t = 0; t < S; ++t) {
              const uint32_t off = b_offset<C>(t, jj, h);
              if (off + 16 > bst.size() || (off & 15)) return 8;
              memcpy(bst.data() + off, &dg[t], 16);
            }
          }
      }
      for (int r = 0; r < g.MT; ++r) {
        memcpy(ast.data(), tiles.data() + (((size_t)r * g.nsteps + ks) * S) * A_BLOCK, C::A_STAGE);
        float* Dr = D.data() + (size_t)r * MROWS * S * BN;
        for (int s = 0; s < S; ++s) {
          const int rows = (S - s) * BN;
          for (int c0 = 0; c0 < rows; c0 += 256) {
            const int n = rows - c0 < 256 ? rows - c0 : 256;
            const uint32_t idesc = tc::idesc_bf16_f32(MROWS, n);
            if ((int)((idesc >> 17) & 63) * 8 != n || (int)((idesc >> 24) & 31) * 16 != MROWS) return 5;
            const uint64_t ad = tc::sdesc_interleave((uint32_t)(s * A_BLOCK * 2), LBO_A, SBO);
            const uint64_t bd = tc::sdesc_interleave((uint32_t)(c0 * 16), C::LBO_B, SBO);
            const uint32_t as = field(ad, 0), al = field(ad, 16), asb = field(ad, 32);
            const uint32_t bs = field(bd, 0), bl = field(bd, 16), bsb = field(bd, 32);
            const int dcol = s * BN + c0;
            if (dcol + n > S * BN) return 9;
            for (int m = 0; m < MROWS; ++m)
              for (int col = 0; col < n; ++col) {
                double sum = 0;
                for (int k = 0; k < 16; ++k) {
                  const uint32_t pa = as + (k >> 3) * al + (m >> 3) * asb + (m & 7) * 16 + (k & 7) * 2;
                  const uint32_t pb = bs + (k >> 3) * bl + (col >> 3) * bsb + (col & 7) * 16 + (k & 7) * 2;
                  if (pa + 2 > ast.size() || pb + 2 > bst.size()) return 6;
                  sum += (double)bf(ast.data() + pa) * (double)bf(bst.data() + pb);
                }
                float& d = Dr[(size_t)m * S * BN + dcol + col];
                d = (float)((ks > 0 || s > 0 ? (double)d : 0.0) + sum);
              }
          }
        }
      }
    }
    for (int r = 0; r < g.MT; ++r)
      for (int m = 0; m < MROWS; ++m) {
        const int n = r * MROWS + m;
        if (n >= g.Nmma) continue;
        for (int jj = 0; jj < BN; ++jj) {
          const int64_t row = row0 + jj;
          if (row >= g.nrows) continue;
          uint32_t gb[C::S];
          for (int gg = 0; gg < S; ++gg)
            memcpy(&gb[gg], &D[((size_t)r * MROWS + m) * S * BN + gg * BN + jj], 4);
          out[row_base(g, row) + (int64_t)n * ksd] = combine<C>(gb, e[jj], em[n]);
        }
      }
    for (int jj = 0; jj < BN; ++jj) {
      const int64_t row = row0 + jj;
      if (row >= g.nrows) continue;
      for (int c = 0; c < g.NX; ++c) out[row_base(g, row) + (int64_t)(g.Nmma + c) * ksd] = xo[(size_t)jj * MAX_NX + c];
    }
  }
  return 0;
}

// emu lcf N nlines cplx bn in.bin M.bin out.bin
static int lcf(int argc, char** argv) {
  if (argc < 9) return 2;
  const int N = atoi(argv[2]);
  const long long nlines = atoll(argv[3]);
  const int cplx = atoi(argv[4]), bn = atoi(argv[5]);
  const size_t cnt = (size_t)nlines * N * (1 + cplx);
  argv += 1;
  double* in = read_exact(argv[5], cnt);
  double* M = read_exact(argv[6], (size_t)N * N);
  int K = 0;
  for (int k = 0; k < N; ++k)
    for (int n = 0; n < N; ++n)
      if (M[(size_t)k * N + n] != 0.0) K = k + 1;
  if (!lc::supported_nk(N, K)) return 3;
  double* out = (double*)malloc(sizeof(double) * cnt);
  for (size_t i = 0; i < cnt; ++i) out[i] = std::numeric_limits<double>::quiet_NaN();
  const int rc = bn == 32 ? lcf_run<lc::CfgNarrow>(lc::make_geom<lc::CfgNarrow>(N, K, nlines, cplx), in, M, out)
                          : lcf_run<lc::CfgWide>(lc::make_geom<lc::CfgWide>(N, K, nlines, cplx), in, M, out);
  if (rc) return rc;
  write_exact(argv[7], out, cnt);
  free(in);
  free(M);
  free(out);
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  std::string mode = argv[1];
  int nm = 0;  // Neumann branch of the Helmholtz programs
  if (mode == "nlu" || mode == "nsolve" || mode == "ncached") {
    nm = 1;
    mode = "h" + mode.substr(1);
  }
  if (mode == "tables") {
    if (argc < 6) return 2;
    LinePlan p;
    HostTables T;
    if (build_plan_host(atoi(argv[2]), atoi(argv[3]), atoi(argv[4]), SGPU_MIXED_DF, p, T) != SGPU_OK) return 3;
    std::vector<double> o;
    for (auto* v : {&T.tw, &T.rk, &T.post})
      for (const cd& c : *v) {
        o.push_back(c.re);
        o.push_back(c.im);
      }
    for (auto* v : {&T.tw_f, &T.rk_f, &T.post_f})
      for (const Cx<df>& c : *v) {
        o.push_back(c.re.hi);
        o.push_back(c.re.lo);
        o.push_back(c.im.hi);
        o.push_back(c.im.lo);
      }
    write_exact(argv[5], o.data(), o.size());
    return 0;
  }
  if (mode == "xform") return xform(argc, argv);
  if (mode == "f256") return f256_mode(argc, argv);
  if (mode == "ozaki" || mode == "ozakic") return ozaki(argc, argv);
  if (mode == "lcf") return lcf(argc, argv);
  if (mode == "lkcheck") {
    // lkcheck: every (line, index) pair of the loop decompositions is visited
    // exactly once for the thread counts the kernels launch with
    const int Ls[] = {1, 2, 4, 8, 16, 32};
    const int ns[] = {1, 2, 7, 16, 129, 257, 300};
    const int nths[] = {1, 32, 128, 256};
    for (int L : Ls)
      for (int n : ns)
        for (int nth : nths)
          for (int rows = 0; rows < 2; ++rows) {
            std::vector<int> hits((size_t)L * n, 0);
            for (int tid = 0; tid < nth; ++tid) {
              LK m = rows ? lk_rows(L, tid, nth) : lk_lines(L, tid, nth);
              SGPU_FOR_LK(m, L, n, c, k) hits[(size_t)c * n + k] += 1;
            }
            for (int h : hits)
              if (h != 1) {
                fprintf(stderr, "lk coverage L=%d n=%d nth=%d rows=%d\n", L, n, nth, rows);
                return 4;
              }
          }
    FILE* f = fopen(argv[2], "wb");
    fclose(f);
    return 0;
  }
  if (mode == "lccombine") {
    // lccombine count groups.bin scales.bin out.bin: the fused contraction's
    // epilogue on n outputs (7 group sums each, integers as doubles; line and
    // column scales as doubles) -> n outputs of combine8, then n of combine
    long long n = atoll(argv[2]);
    if (n % 8) return 2;
    double* gr = read_exact(argv[3], 7 * n);
    double* sc = read_exact(argv[4], 2 * n);
    double* out = (double*)malloc(sizeof(double) * 2 * n);
    typedef lc::CfgWide C;
    for (long long i0 = 0; i0 < n; i0 += 8) {
      uint32_t a[C::S][8];
      int ex[8];
      for (int j = 0; j < 8; ++j) {
        for (int g = 0; g < C::S; ++g) {
          const float f = (float)gr[7 * (i0 + j) + g];
          memcpy(&a[g][j], &f, 4);
        }
        ex[j] = (int)sc[2 * (i0 + j)];
      }
      // combine8 takes one column scale for its eight lines
      const int em = (int)sc[2 * i0 + 1];
      double v[8];
      lc::combine8<C>(a, ex, em, v);
      for (int j = 0; j < 8; ++j) {
        uint32_t gb[C::S];
        for (int g = 0; g < C::S; ++g) gb[g] = a[g][j];
        out[i0 + j] = v[j];
        out[n + i0 + j] = lc::combine<C>(gb, ex[j], em);
      }
    }
    write_exact(argv[5], out, 2 * n);
    return 0;
  }
  if (mode == "dfops") {
    // dfops count x.bin y.bin out.bin -> [round(x), x+y, x-y, x*y] per pair
    long long n = atoll(argv[2]);
    double* x = read_exact(argv[3], n);
    double* y = read_exact(argv[4], n);
    double* out = (double*)malloc(sizeof(double) * 4 * n);
    for (long long i = 0; i < n; ++i) {
      df a = df_from_double(x[i]), b = df_from_double(y[i]);
      out[4 * i] = df_to_double(a);
      out[4 * i + 1] = df_to_double(a + b);
      out[4 * i + 2] = df_to_double(a - b);
      out[4 * i + 3] = df_to_double(a * b);
    }
    write_exact(argv[5], out, 4 * n);
    return 0;
  }
  if (mode == "hlu") {
    long long N = atoll(argv[2]), outer = atoll(argv[3]), inner = atoll(argv[4]);
    long long ns = outer * inner;
    double* a = read_exact(argv[5], ns);
    double* b = read_exact(argv[6], ns);
    std::vector<double*> f(4);
    size_t cnt = (size_t)outer * N * inner;
    double* all = (double*)calloc(4 * cnt, sizeof(double));
    for (int i = 0; i < 4; ++i) f[i] = all + i * cnt;
    for (long long s = 0; s < ns; ++s) helmholtz_lu_prog(N, a, b, nm, f[0], f[1], f[2], f[3], inner, s);
    write_exact(argv[7], all, 4 * cnt);
    return 0;
  }
  if (mode == "hsolve") {
    long long N = atoll(argv[2]), outer = atoll(argv[3]), inner = atoll(argv[4]);
    int dk = atoi(argv[5]);
    size_t cnt = (size_t)outer * N * inner;
    size_t w = dk ? 2 : 1;
    double* b = read_exact(argv[6], cnt * w);
    double* fac = read_exact(argv[7], 4 * cnt);
    double* u = (double*)malloc(sizeof(double) * cnt * w);
    for (size_t i = 0; i < cnt * w; ++i) u[i] = 0.0;
    for (long long s = 0; s < outer * inner; ++s) {
      if (dk)
        helmholtz_solve_prog<cd>((const cd*)b, (cd*)u, nm, fac, fac + cnt, fac + 2 * cnt, fac + 3 * cnt,
                                 N, inner, s);
      else
        helmholtz_solve_prog<double>(b, u, nm, fac, fac + cnt, fac + 2 * cnt, fac + 3 * cnt, N, inner, s);
    }
    write_exact(argv[8], u, cnt * w);
    return 0;
  }
  if (mode == "hcached") {
    // hcached N outer inner data_kind form alfa.bin beta.bin b.bin out.bin
    long long N = atoll(argv[2]), outer = atoll(argv[3]), inner = atoll(argv[4]);
    int dk = atoi(argv[5]), form = atoi(argv[6]);
    long long ns = outer * inner, M = N - 2;
    double* a = read_exact(argv[7], ns);
    double* be = read_exact(argv[8], ns);
    size_t cnt = (size_t)outer * N * inner * (dk ? 2 : 1);
    double* b = read_exact(argv[9], cnt);
    double* u = (double*)malloc(sizeof(double) * cnt);
    for (size_t i = 0; i < cnt; ++i) u[i] = 0.0;
    void* fac = malloc(8 * 4 * (size_t)M * ns);
    for (long long s = 0; s < ns; ++s) {
      if (form >= 2) helmholtz_factor_prog<float>(N, a, be, nm, (float*)fac, ns, s);
      else if (form) helmholtz_factor_prog<df>(N, a, be, nm, (df*)fac, ns, s);
      else helmholtz_factor_prog<double>(N, a, be, nm, (double*)fac, ns, s);
    }
    if (form >= 2) {
      // FP32 sweeps refined by an FP64 (form 2) or double-float (form 3)
      // residual; r is scratch of b's size
      double* r = (double*)malloc(sizeof(double) * cnt);
      for (size_t i = 0; i < cnt; ++i) r[i] = std::numeric_limits<double>::quiet_NaN();
      for (long long t = 0; t < 2 * ns; ++t) {
        long long s = t >> 1;
        int par = (int)(t & 1);
        if (form == 2 && dk) helmholtz_refine_prog<double, cd>((const cd*)b, (cd*)u, (cd*)r, (const float*)fac, a, be, N, inner, ns, s, par, 1e-14, 8);
        else if (form == 2) helmholtz_refine_prog<double, double>(b, u, r, (const float*)fac, a, be, N, inner, ns, s, par, 1e-14, 8);
        else if (dk) helmholtz_refine_prog<df, cd>((const cd*)b, (cd*)u, (cd*)r, (const float*)fac, a, be, N, inner, ns, s, par, 1e-14, 8);
        else helmholtz_refine_prog<df, double>(b, u, r, (const float*)fac, a, be, N, inner, ns, s, par, 1e-14, 8);
      }
      free(r);
      write_exact(argv[10], u, cnt);
      return 0;
    }
    for (long long t = 0; t < 2 * ns; ++t) {
      long long s = t >> 1;
      int par = (int)(t & 1);
      if (form && dk) helmholtz_cached_solve_prog<df, cd>((const cd*)b, (cd*)u, (const df*)fac, nm, N, inner, ns, s, par);
      else if (form) helmholtz_cached_solve_prog<df, double>(b, u, (const df*)fac, nm, N, inner, ns, s, par);
      else if (dk) helmholtz_cached_solve_prog<double, cd>((const cd*)b, (cd*)u, (const double*)fac, nm, N, inner, ns, s, par);
      else helmholtz_cached_solve_prog<double, double>(b, u, (const double*)fac, nm, N, inner, ns, s, par);
    }
    write_exact(argv[10], u, cnt);
    return 0;
  }
  if (mode == "bandsep") {
    // bandsep n nterms gen_term nsys Nb data_kind bands.bin gens.bin coef.bin b.bin out.bin
    // (out: the solution, then the matvec of the solution)
    int n = atoi(argv[2]), nterms = atoi(argv[3]), gen = atoi(argv[4]);
    long long nsys = atoll(argv[5]), Nb = atoll(argv[6]);
    int dk = atoi(argv[7]);
    double* bands = read_exact(argv[8], (size_t)nterms * 5 * n);
    double* gens = read_exact(argv[9], 4 * (size_t)n);
    double* coef = read_exact(argv[10], (size_t)nterms * nsys);
    size_t cnt = (size_t)nsys * Nb * (dk ? 2 : 1);
    double* b = read_exact(argv[11], cnt);
    double* u = (double*)malloc(sizeof(double) * cnt);
    for (size_t i = 0; i < cnt; ++i) u[i] = 0.0;
    const int m = (n + 1) / 2;
    double* fac = (double*)malloc(sizeof(double) * 7 * (size_t)m * 2 * nsys);
    for (size_t i = 0; i < 7 * (size_t)m * 2 * nsys; ++i) fac[i] = std::numeric_limits<double>::quiet_NaN();
    BandSepDesc d{n, nterms, gen, bands, gen >= 0 ? gens : nullptr, coef};
    for (long long ch = 0; ch < 2 * nsys; ++ch) band_sep_factor_prog(d, fac, nsys, ch);
    const double* g = gen >= 0 ? gens : nullptr;
    for (long long ch = 0; ch < 2 * nsys; ++ch) {
      if (dk) band_sep_solve_prog<cd>((const cd*)b, (cd*)u, fac, g, n, Nb, 1, nsys, ch);
      else band_sep_solve_prog<double>(b, u, fac, g, n, Nb, 1, nsys, ch);
    }
    // then the matvec of the solution: out = [u | M u]
    double* mv = (double*)malloc(sizeof(double) * 2 * cnt);
    for (size_t i = 0; i < cnt; ++i) mv[i] = u[i];
    for (size_t i = cnt; i < 2 * cnt; ++i) mv[i] = std::numeric_limits<double>::quiet_NaN();
    for (long long ch = 0; ch < 2 * nsys; ++ch) {
      if (dk) band_sep_matvec_prog<cd>(d, (const cd*)u, (cd*)(mv + cnt), Nb, 1, nsys, ch);
      else band_sep_matvec_prog<double>(d, u, mv + cnt, Nb, 1, nsys, ch);
    }
    write_exact(argv[12], mv, 2 * cnt);
    return 0;
  }
  if (mode == "nmatvec") {
    long long N = atoll(argv[2]), outer = atoll(argv[3]), inner = atoll(argv[4]);
    int dk = atoi(argv[5]);
    size_t cnt = (size_t)outer * N * inner * (dk ? 2 : 1);
    double* v = read_exact(argv[6], cnt);
    double* a = read_exact(argv[7], outer * inner);
    double* be = read_exact(argv[8], outer * inner);
    double* out = (double*)malloc(sizeof(double) * cnt);
    for (size_t i = 0; i < cnt; ++i) out[i] = std::numeric_limits<double>::quiet_NaN();
    for (long long s = 0; s < outer * inner; ++s) {
      if (dk) helmholtz_neumann_matvec_prog<cd>((const cd*)v, (cd*)out, a, be, N, inner, s);
      else helmholtz_neumann_matvec_prog<double>(v, out, a, be, N, inner, s);
    }
    write_exact(argv[9], out, cnt);
    return 0;
  }
  if (mode == "bcapply") {
    // bcapply N outer inner data_kind set_dofs tables u.bin CA.bin alfa.bin CB.bin beta.bin g.bin out.bin
    // tables: bit 0 CA+alfa present, bit 1 CB+beta present
    long long N = atoll(argv[2]), outer = atoll(argv[3]), inner = atoll(argv[4]);
    int dk = atoi(argv[5]), set = atoi(argv[6]), tab = atoi(argv[7]);
    long long ns = outer * inner;
    size_t w = dk ? 2 : 1, cnt = (size_t)outer * N * inner * w;
    double* u = read_exact(argv[8], cnt);
    double* CA = read_exact(argv[9], 2 * (size_t)(N - 2));
    double* al = read_exact(argv[10], ns);
    double* CB = read_exact(argv[11], 2 * (size_t)(N - 2));
    double* be = read_exact(argv[12], ns);
    double* g = read_exact(argv[13], (size_t)outer * 2 * inner * w);
    const double* ca = (tab & 1) ? CA : nullptr;
    const double* cb = (tab & 2) ? CB : nullptr;
    for (long long s = 0; s < ns; ++s) {
      if (dk) bc_apply_prog<cd>((cd*)u, ca, (tab & 1) ? al : nullptr, cb, (tab & 2) ? be : nullptr,
                                (const cd*)g, N, inner, s, set);
      else bc_apply_prog<double>(u, ca, (tab & 1) ? al : nullptr, cb, (tab & 2) ? be : nullptr, g, N,
                                 inner, s, set);
    }
    write_exact(argv[14], u, cnt);
    return 0;
  }
  if (mode == "padd" || mode == "pann") {
    long long N = atoll(argv[2]), outer = atoll(argv[3]), inner = atoll(argv[4]);
    int dk = atoi(argv[5]);
    double scale = atof(argv[6]);
    size_t cnt = (size_t)outer * N * inner * (dk ? 2 : 1);
    double* b = read_exact(argv[7], cnt);
    double* u = (double*)malloc(sizeof(double) * cnt);
    for (size_t i = 0; i < cnt; ++i) u[i] = std::numeric_limits<double>::quiet_NaN();
    for (long long s = 0; s < outer * inner; ++s) {
      if (mode == "padd") {
        if (dk) poisson_add_prog<cd>((const cd*)b, (cd*)u, scale, N, inner, s);
        else poisson_add_prog<double>(b, u, scale, N, inner, s);
      } else {
        if (dk) poisson_ann_prog<cd>((const cd*)b, (cd*)u, scale, 0.0, N, inner, s);
        else poisson_ann_prog<double>(b, u, scale, 0.0, N, inner, s);
      }
    }
    write_exact(argv[8], u, cnt);
    return 0;
  }
  if (mode == "hmatvec") {
    long long N = atoll(argv[2]), outer = atoll(argv[3]), inner = atoll(argv[4]);
    int dk = atoi(argv[5]);
    size_t cnt = (size_t)outer * N * inner;
    size_t w = dk ? 2 : 1;
    double* v = read_exact(argv[6], cnt * w);
    double* a = read_exact(argv[7], outer * inner);
    double* be = read_exact(argv[8], outer * inner);
    double* out = (double*)malloc(sizeof(double) * cnt * w);
    for (long long s = 0; s < outer * inner; ++s) {
      if (dk)
        helmholtz_matvec_prog<cd>((const cd*)v, (cd*)out, a, be, N, inner, s);
      else
        helmholtz_matvec_prog<double>(v, out, a, be, N, inner, s);
    }
    write_exact(argv[9], out, cnt * w);
    return 0;
  }
  if (mode == "banded") {
    // banded n ndiag outer inner data_kind offsets.bin raw.bin u.bin out.bin (LU then solve)
    long long n = atoll(argv[2]);
    int nd = atoi(argv[3]);
    long long outer = atoll(argv[4]), inner = atoll(argv[5]);
    int dk = atoi(argv[6]);
    double* offd = read_exact(argv[7], nd);
    BandDesc b;
    b.nd = nd;
    for (int r = 0; r < nd; ++r) b.off[r] = (int)offd[r];
    double* data = read_exact(argv[8], (size_t)nd * n);
    size_t cnt = (size_t)outer * n * inner * (dk ? 2 : 1);
    double* u = read_exact(argv[9], cnt);
    banded_lu_prog(data, b, n);
    for (long long s = 0; s < outer * inner; ++s) {
      if (dk) banded_solve_prog<cd>((cd*)u, data, b, n, inner, s);
      else banded_solve_prog<double>(u, data, b, n, inner, s);
    }
    write_exact(argv[10], u, cnt);
    return 0;
  }
  if (mode == "bih") {
    // bih outer M inner dk a0 alfa beta sii siu siuu ail aii aiu bill bil bii biu biuu f out
    // (LU, factor_pr, solve; out = u0 u1 u2 l0 l1 ak bk u)
    long long outer = atoll(argv[2]), M = atoll(argv[3]), inner = atoll(argv[4]);
    int dk = atoi(argv[5]);
    double a0 = atof(argv[6]);
    const long long nsys = outer * inner, n = 2 * M, N = n + 4;
    const int w = dk ? 2 : 1;
    double* alfa = read_exact(argv[7], nsys);
    double* beta = read_exact(argv[8], nsys);
    const int shorter[11] = {0, 2, 4, 2, 0, 2, 4, 2, 0, 2, 4};
    double* dg[11];
    for (int q = 0; q < 11; ++q) dg[q] = read_exact(argv[9 + q], n - shorter[q]);
    ref::BihDiags d{dg[0], dg[1], dg[2], dg[3], dg[4], dg[5], dg[6], dg[7], dg[8], dg[9], dg[10]};
    const size_t cnt = (size_t)outer * N * inner * w, fsz = (size_t)2 * nsys * M;
    double* f = read_exact(argv[20], cnt);
    double* fac = (double*)calloc(7 * fsz, sizeof(double));
    double *u0 = fac, *u1 = fac + fsz, *u2 = fac + 2 * fsz, *l0 = fac + 3 * fsz, *l1 = fac + 4 * fsz,
           *ak = fac + 5 * fsz, *bk = fac + 6 * fsz;
    for (long long c = 0; c < 2 * nsys; ++c) ref::bih_lu_chain(c, nsys, d, a0, alfa, beta, u0, u1, u2, l0, l1, M, inner);
    for (long long c = 0; c < 2 * nsys; ++c) ref::bih_factor_pr_chain(c, nsys, ak, bk, l0, l1, M, inner);
    double* u = (double*)malloc(sizeof(double) * cnt);
    memcpy(u, f, sizeof(double) * cnt);
    for (long long c = 0; c < 2 * nsys; ++c) {
      if (dk)
        ref::bih_solve_chain<cd>(c, nsys, (const cd*)f, (cd*)u, u0, u1, u2, l0, l1, ak, bk, a0, N, M, inner);
      else
        ref::bih_solve_chain<double>(c, nsys, f, u, u0, u1, u2, l0, l1, ak, bk, a0, N, M, inner);
    }
    double* out = (double*)malloc(sizeof(double) * (7 * fsz + cnt));
    memcpy(out, fac, sizeof(double) * 7 * fsz);
    memcpy(out + 7 * fsz, u, sizeof(double) * cnt);
    write_exact(argv[21], out, 7 * fsz + cnt);
    return 0;
  }
  if (mode == "bihmv") {
    // bihmv outer N inner dk a0 alfa beta sii .. biuu v out   (M = N - 4)
    long long outer = atoll(argv[2]), N = atoll(argv[3]), inner = atoll(argv[4]);
    int dk = atoi(argv[5]);
    double a0 = atof(argv[6]);
    const long long nsys = outer * inner, M = N - 4;
    const int w = dk ? 2 : 1;
    double* alfa = read_exact(argv[7], nsys);
    double* beta = read_exact(argv[8], nsys);
    const int shorter[11] = {0, 2, 4, 2, 0, 2, 4, 2, 0, 2, 4};
    double* dg[11];
    for (int q = 0; q < 11; ++q) dg[q] = read_exact(argv[9 + q], M - shorter[q]);
    ref::BihDiags d{dg[0], dg[1], dg[2], dg[3], dg[4], dg[5], dg[6], dg[7], dg[8], dg[9], dg[10]};
    const size_t cnt = (size_t)outer * N * inner * w;
    double* v = read_exact(argv[20], cnt);
    double* b = (double*)calloc(cnt, sizeof(double));
    for (long long s2 = 0; s2 < nsys; ++s2) {
      if (dk) ref::bih_matvec_sys<cd>(s2, (const cd*)v, (cd*)b, d, a0, alfa, beta, N, M, inner);
      else ref::bih_matvec_sys<double>(s2, v, b, d, a0, alfa, beta, N, M, inner);
    }
    write_exact(argv[21], b, cnt);
    return 0;
  }
  if (mode == "dma") {
    // dma kind rows cols outer N inner dk per_system skip data u out
    int kind = atoi(argv[2]);
    long long rows = atoll(argv[3]), cols = atoll(argv[4]), outer = atoll(argv[5]), N = atoll(argv[6]),
              inner = atoll(argv[7]);
    int dk = atoi(argv[8]), per = atoi(argv[9]), skip = atoi(argv[10]);
    const long long nsys = outer * inner;
    if (rows < ref::dma_rows(kind) || cols < ref::dma_min_cols(kind) || cols > N) return 4;
    double* data = read_exact(argv[11], (size_t)(per ? nsys : 1) * rows * cols);
    const size_t cnt = (size_t)outer * N * inner * (dk ? 2 : 1);
    double* u = read_exact(argv[12], cnt);
    for (long long s2 = 0; s2 < nsys; ++s2) {
      if (skip && s2 == 0) continue;
      if (dk) ref::dma_solve_sys<cd>(s2, kind, (cd*)u, data, per ? rows * cols : 0, cols, N, inner);
      else ref::dma_solve_sys<double>(s2, kind, u, data, per ? rows * cols : 0, cols, N, inner);
    }
    write_exact(argv[13], u, cnt);
    return 0;
  }
  if (mode == "legrec") {
    // legrec scalar n npts rows cols x w a out
    int scalar = atoi(argv[2]);
    long long n = atoll(argv[3]), npts = atoll(argv[4]);
    int rows = atoi(argv[5]);
    long long cols = atoll(argv[6]);
    if (cols < n + 2 || (rows != 2 && rows != 3)) return 4;
    double* x = read_exact(argv[7], npts);
    double* wv = read_exact(argv[8], npts);
    double* a = read_exact(argv[9], (size_t)rows * cols);
    double* M = (double*)malloc(sizeof(double) * n * npts);
    for (long long j = 0; j < npts; ++j) ref::legendre_matrix_point(j, scalar, x, wv, a, rows, cols, n, npts, M);
    write_exact(argv[10], M, n * npts);
    return 0;
  }
  if (mode == "tdma" || mode == "pdma") {
    long long n = atoll(argv[2]), outer = atoll(argv[3]), inner = atoll(argv[4]);
    int dk = atoi(argv[5]);
    int rows = mode == "tdma" ? 3 : 5;
    double* raw = read_exact(argv[6], rows * n);
    size_t cnt = (size_t)outer * n * inner * (dk ? 2 : 1);
    double* u = read_exact(argv[7], cnt);
    if (mode == "tdma") tdma_lu_prog(raw, n); else pdma_lu_prog(raw, n);
    for (long long s = 0; s < outer * inner; ++s) {
      if (mode == "tdma") {
        if (dk) tdma_solve_prog<cd>((cd*)u, raw, n, inner, s);
        else tdma_solve_prog<double>(u, raw, n, inner, s);
      } else {
        if (dk) pdma_solve_prog<cd>((cd*)u, raw, n, inner, s);
        else pdma_solve_prog<double>(u, raw, n, inner, s);
      }
    }
    write_exact(argv[8], u, cnt);
    return 0;
  }
  return 2;
}
