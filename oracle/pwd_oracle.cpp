// CPU oracle for the plane-wave-destruction (PWD) hot path of pyseistr.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
// calls this file; only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg use it, and only as the checker (or the timed CPU baseline).
//
// This is a restatement, in our own code, of the reference C path
// (pyseistr/src/dip_cfuns.c, sof_cfuns.c, sof3d_cfuns.c, soint3d_cfuns.c),
// templated on the working real type R:
//   R = float  reproduces the reference's float/double mix operation by
//              operation (compile with -ffp-contract=off so that no FMA is
//              formed: the reference is x86-64 SSE code without FMA);
//   R = double is the FP64 oracle: every float of the reference becomes a
//              double, the reference's double arithmetic stays double.
// Every function cites the reference lines it follows.
//
// Parity pin: tests/golden/ holds outputs of the reference itself (compiled
// from its own sources by oracle/Makefile `ref`), generated by
// tests/golden/make_golden.py; tests/test_oracle_golden.py checks this
// restatement against them.

#include <algorithm>
#include <cfenv>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace orc {

enum {
  ORC_OK = 0,
  ORC_EINVAL = 1,
};

// Flags that model the GPU path's arithmetic choices, so the sensitivity of
// the reference algorithm to them can be measured on the CPU.
enum {
  ORC_USUM_DOUBLE = 1,   // line-search residual energies summed in double
  ORC_FILTER_REAL = 2,   // all-pass filter products in R instead of double
  ORC_TRI_CHUNK = 4,     // triangle running sums as a 32-element chunked scan
  ORC_FILTER_FF = 8,     // filter products in float-float (pair) arithmetic
  ORC_TRI_EXACT = 16,    // triangle smoothing evaluated in double, rounded once
  ORC_GPU_DOTS = 32,     // dot products and residual energies summed in the
                         // GPU plain path's order (see gpuorder::dot)
  ORC_TRUE_RESIDUAL = 512,  // CG residual formed as W x - dat each iteration
                            // and sr as W sx, instead of their recurrences
};

// Float-float helpers (Dekker / Knuth error-free transformations) used by
// the ORC_FILTER_FF model of the GPU filter evaluation.
struct FF {
  float h, l;
};
static inline FF ff_quick(float a, float b) {
  float s = a + b;
  return {s, b - (s - a)};
}
static inline FF ff_two_prod(float a, float b) {
  float p = a * b;
  return {p, std::fma(a, b, -p)};
}
static inline FF ff_mul_f(FF a, float b) {
  FF p = ff_two_prod(a.h, b);
  float e = std::fma(a.l, b, p.l);
  return ff_quick(p.h, e);
}
static inline FF ff_mul(FF a, FF b) {
  FF p = ff_two_prod(a.h, b.h);
  float e = std::fma(a.h, b.l, std::fma(a.l, b.h, p.l));
  return ff_quick(p.h, e);
}
static inline FF ff_add(FF a, FF b) {
  float s = a.h + b.h;
  float bb = s - a.h;
  float e = (a.h - (s - bb)) + (b.h - bb);
  e += a.l + b.l;
  return ff_quick(s, e);
}
static inline FF ff_from_double(double x) {
  float h = (float)x;
  return {h, (float)(x - (double)h)};
}

// ---------------------------------------------------------------------------
// All-pass (Thiran) filter coefficients.
// apfilt_init  dip_cfuns.c:835-855 ; passfilter :863-881 ; aderfilter :883-910
// ---------------------------------------------------------------------------
template <class R>
struct ApFilter {
  int nf = 0;
  double b[17];
  bool real_products = false;  // ORC_FILTER_REAL
  bool ff_products = false;    // ORC_FILTER_FF (float instantiation only)

  void init(int nw) {
    nf = 2 * nw;
    for (int k = 0; k <= nf; k++) {
      double bk = 1.0;
      for (int j = 0; j < nf; j++) {
        if (j < nf - k)
          bk *= (k + j + 1.0) / (2 * (2 * j + 1) * (j + 1));
        else
          bk *= 1.0 / (2 * (2 * j + 1));
      }
      b[k] = bk;
    }
  }

  // Factor of the product for tap k, index j: (nf-j-p) or ((p+j)+1), both
  // evaluated in the working precision exactly as the C expression does.
  inline R factor(int k, int j, R p) const {
    if (j < nf - k) return (R)(nf - j) - p;
    R t = p + (R)j;
    return t + (R)1;
  }

  void pass(R p, R* a) const {
    for (int k = 0; k <= nf; k++) {
      if (ff_products) {
        FF ak = ff_from_double(b[k]);
        for (int j = 0; j < nf; j++) ak = ff_mul_f(ak, (float)factor(k, j, p));
        a[k] = (R)(ak.h + ak.l);
      } else if (real_products) {
        R ak = (R)b[k];
        for (int j = 0; j < nf; j++) ak = ak * factor(k, j, p);
        a[k] = ak;
      } else {
        double ak = b[k];
        for (int j = 0; j < nf; j++) ak *= (double)factor(k, j, p);
        a[k] = (R)ak;
      }
    }
  }

  void ader(R p, R* a) const {
    for (int k = 0; k <= nf; k++) {
      if (ff_products) {
        FF ak = {0.f, 0.f};
        for (int i = 0; i < nf; i++) {
          FF ai = {-1.f, 0.f};
          for (int j = 0; j < nf; j++) {
            if (j != i)
              ai = ff_mul_f(ai, (float)factor(k, j, p));
            else if (j < nf - k)
              ai = {-ai.h, -ai.l};
          }
          ak = ff_add(ak, ai);
        }
        FF r = ff_mul(ak, ff_from_double(b[k]));
        a[k] = (R)(r.h + r.l);
      } else if (real_products) {
        R ak = 0;
        for (int i = 0; i < nf; i++) {
          R ai = -1;
          for (int j = 0; j < nf; j++) {
            if (j != i)
              ai = ai * factor(k, j, p);
            else if (j < nf - k)
              ai = -ai;
          }
          ak = ak + ai;
        }
        a[k] = ak * (R)b[k];
      } else {
        double ak = 0.;
        for (int i = 0; i < nf; i++) {
          double ai = -1.0;
          for (int j = 0; j < nf; j++) {
            if (j != i)
              ai *= (double)factor(k, j, p);
            else if (j < nf - k)
              ai *= (-1);
          }
          ak += ai;
        }
        a[k] = (R)(ak * b[k]);
      }
    }
  }
};

// ---------------------------------------------------------------------------
// BLAS-1 helpers, dip_cfuns.c:122-209.
// ---------------------------------------------------------------------------
template <class R>
static double dsdot(long n, const R* x, const R* y) {
  double dot = 0.;
  for (long i = 0; i < n; i++) dot += (double)x[i] * y[i];
  return dot;
}

// The GPU plain path's summation order for a dot product of float vectors
// (pyseistr_gb300/csrc/pwd_dip.cu sec_sum_last, pwd_common.cuh ffacc and
// block_sum): the section is cut into tiles of 8192 samples; in a tile,
// thread j of 256 accumulates samples j, j+256, ... as a float-float pair
// (error-free product and two-sum), converts it to double (h + l), and the
// block sums its threads by the warp shuffle-down tree (offsets 16..1, then
// the 8 warp sums by the same tree); the last tile then has thread j sum the
// tile partials j, j+256, ... in double, in tile order, and reduces those
// 256 values by the same block tree.  Model of the GPU only (to show which
// of its results differ from the reference by summation order alone).
namespace gpuorder {
constexpr long kTile = 8192;
constexpr int kThreads = 256;
static inline void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
static double tree32(double* v) {  // lane 0 of a shuffle-down tree
  for (int o = 16; o > 0; o >>= 1)
    for (int l = 0; l < o; l++) v[l] = v[l] + v[l + o];
  return v[0];
}
static double block_sum(const double* t) {  // 256 thread values
  double w[32];
  for (int k = 0; k < 32; k++) w[k] = 0.0;
  for (int wi = 0; wi < kThreads / 32; wi++) {
    double v[32];
    for (int l = 0; l < 32; l++) v[l] = t[wi * 32 + l];
    w[wi] = tree32(v);
  }
  return tree32(w);
}
static double dot(long n, const float* x, const float* y) {
  const long ntile = (n + kTile - 1) / kTile;
  std::vector<double> part(ntile);
  double tv[kThreads];
  for (long t = 0; t < ntile; t++) {
    const long lo = t * kTile, hi = std::min(n, lo + kTile);
    for (int j = 0; j < kThreads; j++) {
      float h = 0.f, l = 0.f;
      for (long i = lo + j; i < hi; i += kThreads) {
        const float p = x[i] * y[i];
        const float pe = std::fma(x[i], y[i], -p);
        float sh, sl;
        two_sum(h, p, sh, sl);
        h = sh;
        l = l + (sl + pe);
      }
      tv[j] = (double)h + (double)l;
    }
    part[t] = block_sum(tv);
  }
  for (int j = 0; j < kThreads; j++) {
    double v = 0.0;
    for (long i = j; i < ntile; i += kThreads) v += part[i];
    tv[j] = v;
  }
  return block_sum(tv);
}
}  // namespace gpuorder

static bool g_gpu_dots = false;  // ORC_GPU_DOTS for the float dip path
static int g_store16 = 0;        // spray factor-store precision model (0 off, 1 FP16, 2 BF16)
static int g_cg_store16 = 0;     // CG direction-store precision model (same codes)
static float round16(float x) {
  if (g_store16 == 1) return (float)(_Float16)x;
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return x;
  u += 0x7fffu + ((u >> 16) & 1u);
  u &= 0xffff0000u;
  float y;
  std::memcpy(&y, &u, 4);
  return y;
}

template <class R>
static double dsdot_dip(long n, const R* x, const R* y) {
  if constexpr (sizeof(R) == 4) {
    if (g_gpu_dots) return gpuorder::dot(n, (const float*)x, (const float*)y);
  }
  return dsdot(n, x, y);
}

template <class R>
static void saxpy(long n, R a, const R* x, R* y) {
  for (long i = 0; i < n; i++) y[i] += a * x[i];
}
template <class R>
static R snrm2(long n, const R* x) {  // sum of squares, as the reference
  R xn = 0;
  for (long i = 0; i < n; i++) xn += x[i] * x[i];
  return xn;
}

// ---------------------------------------------------------------------------
// Triangle smoothing (adjoint form used by divne), dip_cfuns.c:405-625.
// ---------------------------------------------------------------------------
template <class R>
struct Triangle {
  int nx, nb, np;
  R wt;
  std::vector<R> tmp;
  void init(int nbox, int ndat) {  // ps_triangle_init :405-428 (box=false)
    nx = ndat;
    nb = nbox;
    np = ndat + 2 * nbox;
    wt = (R)(1.0 / (nbox * nbox));
    tmp.assign(np, (R)0);
  }
  // triple2 :564-580 (box=false)
  void triple2(long o, long d, const R* x) {
    for (int i = 0; i < np; i++) tmp[i] = 0;
    R a0 = -wt, a1 = (R)(2. * wt), a2 = -wt;
    for (int i = 0; i < nx; i++) tmp[i] += a0 * x[o + i * d];
    for (int i = 0; i < nx; i++) tmp[nb + i] += a1 * x[o + i * d];
    for (int i = 0; i < nx; i++) tmp[2 * nb + i] += a2 * x[o + i * d];
  }
  bool chunked = false;  // ORC_TRI_CHUNK model
  void scan_chunked(bool fwd) {
    const int C = 32;
    R carry = 0;
    if (fwd) {
      for (int c0 = 0; c0 < np; c0 += C) {
        R s = 0, tot;
        int c1 = std::min(np, c0 + C);
        for (int i = c0; i < c1; i++) { s += tmp[i]; tmp[i] = s; }
        tot = s;
        for (int i = c0; i < c1; i++) tmp[i] = carry + tmp[i];
        carry = carry + tot;
      }
    } else {
      for (int c1 = np; c1 > 0; c1 -= C) {
        int c0 = std::max(0, c1 - C);
        R s = 0, tot;
        for (int i = c1 - 1; i >= c0; i--) { s += tmp[i]; tmp[i] = s; }
        tot = s;
        for (int i = c0; i < c1; i++) tmp[i] = carry + tmp[i];
        carry = carry + tot;
      }
    }
  }
  // doubint2 :508-529 (der=false)
  void doubint2() {
    if (chunked) { scan_chunked(true); scan_chunked(false); return; }
    R t = 0;
    for (int i = 0; i < np; i++) {
      t += tmp[i];
      tmp[i] = t;
    }
    t = 0;
    for (int i = np - 1; i >= 0; i--) {
      t += tmp[i];
      tmp[i] = t;
    }
  }
  // fold2 :458-484
  void fold2(long o, long d, R* x) const {
    int i, j;
    for (i = 0; i < nx; i++) x[o + i * d] = tmp[i + nb];
    for (j = nb + nx; j < np; j += nx) {
      for (i = 0; i < nx && i < np - j; i++) x[o + (nx - 1 - i) * d] += tmp[j + i];
      j += nx;
      for (i = 0; i < nx && i < np - j; i++) x[o + i * d] += tmp[j + i];
    }
    for (j = nb; j >= 0; j -= nx) {
      for (i = 0; i < nx && i < j; i++) x[o + i * d] += tmp[j - 1 - i];
      j -= nx;
      for (i = 0; i < nx && i < j; i++) x[o + (nx - 1 - i) * d] += tmp[j - 1 - i];
    }
  }
  // ps_smooth2 :616-625
  bool exact = false;  // ORC_TRI_EXACT model (the GPU mixed mode's smoothing)
  void smooth2(long o, long d, R* x) {
    if (exact) {
      // the same spread, sums and fold in double, each output rounded once
      std::vector<double> t(np, 0.0);
      const double w = 1.0 / ((double)nb * nb);
      for (int i = 0; i < nx; i++) {
        const double xi = (double)x[o + i * d];
        t[i] -= w * xi;
        t[nb + i] += 2.0 * w * xi;
        t[2 * nb + i] -= w * xi;
      }
      double a = 0;
      for (int i = 0; i < np; i++) { a += t[i]; t[i] = a; }
      a = 0;
      for (int i = np - 1; i >= 0; i--) { a += t[i]; t[i] = a; }
      std::vector<double> y(nx);
      for (int i = 0; i < nx; i++) y[i] = t[i + nb];
      int i, j;
      for (j = nb + nx; j < np; j += nx) {
        for (i = 0; i < nx && i < np - j; i++) y[nx - 1 - i] += t[j + i];
        j += nx;
        for (i = 0; i < nx && i < np - j; i++) y[i] += t[j + i];
      }
      for (j = nb; j >= 0; j -= nx) {
        for (i = 0; i < nx && i < j; i++) y[i] += t[j - 1 - i];
        j -= nx;
        for (i = 0; i < nx && i < j; i++) y[nx - 1 - i] += t[j - 1 - i];
      }
      for (i = 0; i < nx; i++) x[o + i * d] = (R)y[i];
      return;
    }
    triple2(o, d, x);
    doubint2();
    fold2(o, d, x);
  }
};

// ps_first_index dip_cfuns.c:99-119
static long first_index(int i, long j, int dim, const int* n, const long* s) {
  long n123 = 1, i0 = 0;
  for (int k = 0; k < dim; k++) {
    if (k == i) continue;
    long ii = (j / n123) % n[k];
    n123 *= n[k];
    i0 += ii * s[k];
  }
  return i0;
}

// N-D triangle smoother as a linear operator, ps_trianglen_* :650-712.
template <class R>
struct TriangleN {
  int dim = 3;
  int n[3];
  long s[3];
  long nd;
  bool on[3];
  Triangle<R> tr[3];
  std::vector<R> tmp;
  void init(const int* nbox, const int* ndat) {
    nd = 1;
    for (int i = 0; i < dim; i++) {
      on[i] = nbox[i] > 1;
      if (on[i]) tr[i].init(nbox[i], ndat[i]);
      s[i] = nd;
      n[i] = ndat[i];
      nd *= ndat[i];
    }
    tmp.assign(nd, (R)0);
  }
  // trianglen_lop :672-712 ; the same smoothing serves adjoint and forward
  void lop(bool adj, bool add, R* x, R* y) {
    if (!add) {
      R* z = adj ? x : y;
      for (long i = 0; i < nd; i++) z[i] = 0;
    }
    const R* src = adj ? y : x;
    for (long i = 0; i < nd; i++) tmp[i] = src[i];
    for (int i = 0; i < dim; i++) {
      if (!on[i]) continue;
      long nl = nd / n[i];
      for (long j = 0; j < nl; j++) {
        long i0 = first_index(i, j, dim, n, s);
        tr[i].smooth2(i0, s[i], tmp.data());
      }
    }
    R* dst = adj ? x : y;
    for (long i = 0; i < nd; i++) dst[i] += tmp[i];
  }
};

// ---------------------------------------------------------------------------
// Shaping-regularised CG (prec=NULL, hasp0=false), ps_conjgrad :257-383,
// with oper = ps_weight_lop (:739-758) and shape = trianglen_lop.
// ---------------------------------------------------------------------------
template <class R>
struct ConjGrad {
  long n;
  R eps;  // eps1*eps1 with eps1 = 1 (ps_divn_init :777)
  R tol;
  std::vector<R> r, sp, gp, sx, gx, sr, gr;
  void init(long n_, R eps1, R tol1) {
    n = n_;
    eps = eps1 * eps1;
    tol = tol1;
    r.assign(n, 0); sp.assign(n, 0); gp.assign(n, 0); sx.assign(n, 0);
    gx.assign(n, 0); sr.assign(n, 0); gr.assign(n, 0);
  }
  bool true_residual = false;  // ORC_TRUE_RESIDUAL precision model
  // returns the number of iterations run (for diagnostics)
  int solve(TriangleN<R>& S, const R* w, R* p, R* x, const R* dat, int niter) {
    double gn, gnp = 0., alpha, beta, g0 = 0., dg = 0., r0;
    for (long i = 0; i < n; i++) r[i] = -dat[i];
    for (long i = 0; i < n; i++) p[i] = 0;
    for (long i = 0; i < n; i++) x[i] = 0;
    r0 = dsdot_dip(n, r.data(), r.data());
    if (r0 == 0.) return 0;
    int iter;
    for (iter = 0; iter < niter; iter++) {
      for (long i = 0; i < n; i++) gp[i] = eps * p[i];
      if (true_residual) {  // precision model: r = W x - dat formed afresh, one rounding
        for (long i = 0; i < n; i++) r[i] = (R)((double)w[i] * (double)x[i] - (double)dat[i]);
      }
      for (long i = 0; i < n; i++) gx[i] = -eps * x[i];
      for (long i = 0; i < n; i++) gx[i] += r[i] * w[i];  // W' r (add)
      S.lop(true, true, gp.data(), gx.data());              // gp += S' gx
      S.lop(false, false, gp.data(), gx.data());            // gx = S gp
      for (long i = 0; i < n; i++) gr[i] = (R)0 + gx[i] * w[i];  // gr = W gx
      gn = dsdot_dip(n, gp.data(), gp.data());
      if (iter == 0) {
        g0 = gn;
        sp = gp; sx = gx; sr = gr;
      } else {
        alpha = gn / gnp;
        dg = gn / g0;
        if (alpha < (double)tol || dg < (double)tol) break;
        R a = (R)alpha;
        saxpy(n, a, sp.data(), gp.data()); std::swap(sp, gp);
        saxpy(n, a, sx.data(), gx.data()); std::swap(sx, gx);
        saxpy(n, a, sr.data(), gr.data()); std::swap(sr, gr);
      }
      if (g_cg_store16) {  // precision model: the conjugate directions stored in 16 bits
        const int keep = g_store16;
        g_store16 = g_cg_store16;
        for (auto* v : {&sp, &sx, &sr})
          for (auto& e : *v) e = (R)round16((float)e);
        g_store16 = keep;
      }
      if (true_residual)  // sr = W sx (its value in exact arithmetic)
        for (long i = 0; i < n; i++) sr[i] = w[i] * sx[i];
      beta = dsdot_dip(n, sr.data(), sr.data()) +
             (double)eps * (dsdot_dip(n, sp.data(), sp.data()) - dsdot_dip(n, sx.data(), sx.data()));
      alpha = -gn / beta;
      R a = (R)alpha;
      saxpy(n, a, sp.data(), p);
      saxpy(n, a, sx.data(), x);
      saxpy(n, a, sr.data(), r.data());
      gnp = gn;
    }
    return iter;
  }
};

// ps_divne :796-827 ; eps is the file-scope CG eps (=1, quirk Q1)
template <class R>
static void divne(ConjGrad<R>& cg, TriangleN<R>& S, std::vector<R>& pbuf, R* num, R* den,
                  R* rat, R eps, int niter) {
  long n = cg.n;
  double norm;
  if (eps > (R)0) {
    for (long i = 0; i < n; i++) {
      norm = 1.0 / std::hypot((double)den[i], (double)eps);
      num[i] = (R)(num[i] * norm);
      den[i] = (R)(den[i] * norm);
    }
  }
  norm = dsdot_dip(n, den, den);
  if (norm == 0.0) {
    for (long i = 0; i < n; i++) rat[i] = 0;
    return;
  }
  norm = std::sqrt(n / norm);
  for (long i = 0; i < n; i++) {
    num[i] = (R)(num[i] * norm);
    den[i] = (R)(den[i] * norm);
  }
  cg.solve(S, den, pbuf.data(), rat, num, niter);
}

// ---------------------------------------------------------------------------
// Plane-wave destruction residual, allpass1 (:1135-1200, inline, neighbour
// +n1) and allpass2 (:1399-1465, crossline, neighbour +n1*n2); left=false,
// drift=false, nj=1 as dipc hard-codes (:1727-1786).
// ---------------------------------------------------------------------------
template <class R>
static void allpass(int dip, bool der, const ApFilter<R>& af, int nw, int nx, int ny,
                    int nz, const R* xx, const R* pp, R* yy) {
  long n = (long)nx * ny * nz;
  for (long i = 0; i < n; i++) yy[i] = 0;
  long ip = (dip == 1) ? nx : (long)nx * ny;
  int iy1 = (dip == 1) ? ny - 1 : ny;
  int iz1 = (dip == 1) ? nz : nz - 1;
  R flt[17];
  for (int iz = 0; iz < iz1; iz++)
    for (int iy = 0; iy < iy1; iy++)
      for (int ix = nw; ix < nx - nw; ix++) {
        long i = ix + (long)nx * (iy + (long)ny * iz);
        if (der)
          af.ader(pp[i], flt);
        else
          af.pass(pp[i], flt);
        for (int iw = 0; iw <= 2 * nw; iw++) {
          int is = iw - nw;
          yy[i] += (xx[i + is + ip] - xx[i - is]) * flt[iw];
        }
      }
}

// mask32 :914-997 with both=false, nj1=nj2=1.  m0: inline, m1: crossline.
template <class R>
static void mask32(int nw, int nx, int ny, int nz, const R* yy, std::vector<uint8_t>& m0,
                   std::vector<uint8_t>& m1) {
  long n = (long)nx * ny * nz;
  std::vector<uint8_t> xx(n);
  m0.assign(n, 0);
  m1.assign(n, 0);
  for (long i = 0; i < n; i++) xx[i] = (yy[i] == (R)0);
  for (int iz = 0; iz < nz; iz++)
    for (int iy = 0; iy < ny - 1; iy++)
      for (int ix = nw; ix < nx - nw; ix++) {
        long i = ix + (long)nx * (iy + (long)ny * iz);
        for (int iw = 0; iw <= 2 * nw; iw++) {
          int is = iw - nw;
          m0[i] = m0[i] || xx[i - is] || xx[i + nx + is];
        }
      }
  for (int iz = 0; iz < nz - 1; iz++)
    for (int iy = 0; iy < ny; iy++)
      for (int ix = nw; ix < nx - nw; ix++) {
        long i = ix + (long)nx * (iy + (long)ny * iz);
        for (int iw = 0; iw <= 2 * nw; iw++) {
          int is = iw - nw;
          m1[i] = m1[i] || xx[i - is] || xx[i + (long)ny * nx + is];
        }
      }
}

// State of one dip estimation (dip3_init :1585-1608 + ps_divn_init :765-779).
template <class R>
struct DipState {
  int n1, n2, n3;
  long nd;
  std::vector<R> u1, u2, dp, p0, pbuf;
  TriangleN<R> tri;
  ConjGrad<R> cg;
  ApFilter<R> af;
  int flags = 0;
  void init(int m1, int m2, int m3, const int* rect) {
    n1 = m1; n2 = m2; n3 = m3;
    nd = (long)n1 * n2 * n3;
    u1.assign(nd, 0); u2.assign(nd, 0); dp.assign(nd, 0); p0.assign(nd, 0);
    pbuf.assign(nd, 0);
    int nn[3] = {n1, n2, n3};
    int rr[3] = {rect[0], rect[1], rect[2]};
    tri.init(rr, nn);
    cg.init(nd, (R)1., (R)1.e-6);
  }
  // Residual energy: float serial sum as the reference (:1653, :1681), or
  // the double sum the GPU path uses (ORC_USUM_DOUBLE).
  double energy(const R* v) const {
    if (flags & (ORC_USUM_DOUBLE | ORC_GPU_DOTS)) return dsdot_dip(nd, v, v);
    R s = 0;
    for (long i = 0; i < nd; i++) s += v[i] * v[i];
    return (double)s;
  }
  // dip3 :1619-1691 (left=false, nj=1, drift=false); ls[iter] receives the
  // number of line-search trials the iteration ran (diagnostics).
  void dip3(int dip, int niter, int liter, int nw, const R* u, R* p, const uint8_t* mask,
            R pmin, R pmax, int* ls) {
    af.init(nw);
    af.real_products = (flags & ORC_FILTER_REAL) != 0;
    af.ff_products = (flags & ORC_FILTER_FF) != 0 && sizeof(R) == 4;
    for (int i = 0; i < 3; i++) {
      tri.tr[i].chunked = (flags & ORC_TRI_CHUNK) != 0;
      tri.tr[i].exact = (flags & ORC_TRI_EXACT) != 0;
    }
    cg.true_residual = (flags & ORC_TRUE_RESIDUAL) != 0;
    allpass(dip, false, af, nw, n1, n2, n3, u, p, u2.data());
    for (int iter = 0; iter < niter; iter++) {
      allpass(dip, true, af, nw, n1, n2, n3, u, p, u1.data());
      for (long i = 0; i < nd; i++) p0[i] = p[i];
      double usum = energy(u2.data());
      if (mask) {
        for (long i = 0; i < nd; i++)
          if (mask[i]) { u1[i] = 0; u2[i] = 0; }
      }
      divne(cg, tri, pbuf, u2.data(), u1.data(), dp.data(), cg.eps, liter);
      R lam = 1;
      int k;
      for (k = 0; k < 8; k++) {
        for (long i = 0; i < nd; i++) {
          R pi = p0[i] + lam * dp[i];
          if (pi < pmin) pi = pmin;
          if (pi > pmax) pi = pmax;
          p[i] = pi;
        }
        allpass(dip, false, af, nw, n1, n2, n3, u, p, u2.data());
        double usum2 = energy(u2.data());
        if (usum2 < usum) break;
        lam *= (R)0.5;
      }
      if (ls) ls[iter] = k < 8 ? k + 1 : 8;
    }
  }
};

// dipc :1694-1989.  Output: n (2D, n3==1) or 2n (3D: inline then crossline).
template <class R>
static int dipc(const R* u, const R* maskdata, R* pout, int n1, int n2, int n3, int niter,
                int liter, int order, const int* rect, int flags, int* ls) {
  if (n1 < 1 || n2 < 1 || n3 < 1 || order < 1 || order > 8 || niter < 0 || liter < 0)
    return ORC_EINVAL;
  long n = (long)n1 * n2 * n3;
  int n4 = (n3 == 1) ? 0 : 2;
  DipState<R> st;
  st.flags = flags;
  g_gpu_dots = (flags & ORC_GPU_DOTS) != 0;
  st.init(n1, n2, n3, rect);
  std::vector<uint8_t> m0, m1;
  if (maskdata) mask32(order, n1, n2, n3, maskdata, m0, m1);
  R pmin = (R)-FLT_MAX, pmax = (R)FLT_MAX;
  for (long i = 0; i < n; i++) pout[i] = 0;
  st.dip3(1, niter, liter, order, u, pout, maskdata ? m0.data() : nullptr, pmin, pmax, ls);
  if (n4 != 0) {
    for (long i = 0; i < n; i++) pout[n + i] = 0;
    st.dip3(2, niter, liter, order, u, pout + n, maskdata ? m1.data() : nullptr, pmin, pmax,
            ls ? ls + niter : nullptr);
  }
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// Banded LDL' solver, sf_banded_* sof_cfuns.c:137-307.
// ---------------------------------------------------------------------------
template <class R>
struct Banded {
  int n, band;
  std::vector<R> d;
  std::vector<std::vector<R>> o;
  void init(int n_, int band_) {
    n = n_;
    band = band_;
    o.resize(band);
    for (int i = 0; i < band; i++) o[i].assign(std::max(n - 1 - i, 1), 0);
    d.assign(n, 0);
  }
  void define(const R* diag, const std::vector<std::vector<R>>& offd) {
    for (int k = 0; k < n; k++) {
      R t = diag[k];
      int m1 = std::min(k, band);
      for (int m = 0; m < m1; m++) t -= o[m][k - m - 1] * o[m][k - m - 1] * d[k - m - 1];
      d[k] = t;
      int nn1 = std::min(n - k - 1, band);
      for (int q = 0; q < nn1; q++) {
        t = offd[q][k];
        m1 = std::min(k, band - q - 1);
        for (int m = 0; m < m1; m++) t -= o[m][k - m - 1] * o[q + m + 1][k - m - 1] * d[k - m - 1];
        o[q][k] = t / d[k];
      }
    }
  }
  void solve(R* b) const {
    for (int k = 1; k < n; k++) {
      R t = b[k];
      int m1 = std::min(k, band);
      for (int m = 0; m < m1; m++) t -= o[m][k - m - 1] * b[k - m - 1];
      b[k] = t;
    }
    for (int k = n - 1; k >= 0; k--) {
      R t = b[k] / d[k];
      int m1 = std::min(n - k - 1, band);
      for (int m = 0; m < m1; m++) t -= o[m][k] * b[k + m + 1];
      b[k] = t;
    }
  }
};

// PWD matrix, pwd_* sof_cfuns.c:415-555.
template <class R>
struct Pwd {
  int n, na;
  std::vector<std::vector<R>> a;
  std::vector<R> bb;
  ApFilter<R> af;
  void init(int n1, int nw) {
    n = n1;
    na = 2 * nw + 1;
    a.assign(na, std::vector<R>(n1, 0));
    bb.assign(na, 0);
    af.init(nw);
  }
  // pwd_define :453-497
  void define(bool adj, const R* pp, R* diag, std::vector<std::vector<R>>& offd) {
    int nw = (na - 1) / 2;
    for (int i = 0; i < n; i++) {
      af.pass(pp[i], bb.data());
      for (int j = 0; j < na; j++) a[j][i] = adj ? bb[na - 1 - j] : bb[j];
    }
    for (int i = 0; i < n; i++) {
      for (int j = 0; j < na; j++) {
        int k = i + j - nw;
        if (k >= nw && k < n - nw) {
          R aj = a[j][k];
          diag[i] += aj * aj;
        }
      }
      for (int m = 0; m < 2 * nw; m++)
        for (int j = m + 1; j < na; j++) {
          int k = i + j - nw;
          if (k >= nw && k < n - nw) {
            R aj = a[j][k];
            R am = a[j - m - 1][k];
            offd[m][i] += am * aj;
          }
        }
    }
  }
  // pwd_set :499-555 (inp, out and tmp may alias as in the reference)
  void set(bool adj, R* inp, R* out, R* tmp) const {
    int nw = (na - 1) / 2;
    if (adj) {
      for (int i = 0; i < n; i++) tmp[i] = 0;
      for (int i = 0; i < n; i++)
        for (int j = 0; j < na; j++) {
          int k = i + j - nw;
          if (k >= nw && k < n - nw) tmp[k] += a[j][k] * out[i];
        }
      for (int i = 0; i < n; i++) inp[i] = 0;
      for (int i = nw; i < n - nw; i++)
        for (int j = 0; j < na; j++) {
          int k = i + j - nw;
          inp[k] += a[j][i] * tmp[i];
        }
    } else {
      for (int i = 0; i < n; i++) tmp[i] = 0;
      for (int i = nw; i < n - nw; i++)
        for (int j = 0; j < na; j++) {
          int k = i + j - nw;
          tmp[i] += a[j][i] * inp[k];
        }
      for (int i = 0; i < n; i++) {
        out[i] = 0;
        for (int j = 0; j < na; j++) {
          int k = i + j - nw;
          if (k >= nw && k < n - nw) out[i] += a[j][k] * tmp[k];
        }
      }
    }
  }
};

// Trace prediction, predict_* sof_cfuns.c:558-649 and sof3d_cfuns.c:501-661.
template <class R>
struct Predict {
  int n1, nb;
  R eps, eps2;
  Banded<R> slv;
  std::vector<R> diag;
  std::vector<std::vector<R>> offd;
  Pwd<R> w1, w2;
  void init(int nt, R e, int nw, bool two) {  // predict_init :566-589 / :509-534
    n1 = nt;
    nb = 2 * nw;
    eps = e;
    eps2 = e;
    slv.init(n1, nb);
    diag.assign(n1, 0);
    offd.assign(nb, std::vector<R>(n1, 0));
    w1.init(n1, nw);
    if (two) w2.init(n1, nw);
  }
  // Precision model of a factor store kept in 16 bits (g_store16: 1 FP16,
  // 2 BF16): the taps the filter application reads and the LDL' factors the
  // solves read rounded to 16 bits; the band itself is formed from the
  // exact taps, as a factor kernel would.
  void store16() {
    for (auto& col : w1.a)
      for (auto& v : col) v = (R)round16((float)v);
    for (auto& v : slv.d) v = (R)round16((float)v);
    for (auto& col : slv.o)
      for (auto& v : col) v = (R)round16((float)v);
  }
  // regularization :603-620
  void regularization() {
    for (int i1 = 0; i1 < n1; i1++) {
      diag[i1] = (R)(6. * eps);
      offd[0][i1] = (R)(-4. * eps);
      offd[1][i1] = eps;
      for (int ib = 2; ib < nb; ib++) offd[ib][i1] = 0;
    }
    diag[0] = diag[n1 - 1] = eps2 + eps;
    diag[1] = diag[n1 - 2] = (R)(eps2 + 5. * eps);
    offd[0][0] = offd[0][n1 - 2] = (R)(-2. * eps);
  }
  // predict_step :622-649
  void step(bool adj, bool forw, R* trace, const R* pp) {
    regularization();
    w1.define(forw, pp, diag.data(), offd);
    slv.define(diag.data(), offd);
    if (g_store16) store16();
    if (adj) slv.solve(trace);
    R t0 = trace[0], t1 = trace[1], t2 = trace[n1 - 2], t3 = trace[n1 - 1];
    w1.set(adj, trace, trace, diag.data());
    trace[0] += eps2 * t0;
    trace[1] += eps2 * t1;
    trace[n1 - 2] += eps2 * t2;
    trace[n1 - 1] += eps2 * t3;
    if (!adj) slv.solve(trace);
  }
  // predict1_step sof3d_cfuns.c:596-622
  void step1(bool forw, R* trace1, const R* pp, R* trace) {
    regularization();
    w1.define(forw, pp, diag.data(), offd);
    slv.define(diag.data(), offd);
    R t0 = trace1[0], t1 = trace1[1], t2 = trace1[n1 - 2], t3 = trace1[n1 - 1];
    w1.set(false, trace1, trace, diag.data());
    trace[0] += eps2 * t0;
    trace[1] += eps2 * t1;
    trace[n1 - 2] += eps2 * t2;
    trace[n1 - 1] += eps2 * t3;
    slv.solve(trace);
  }
  // predict2_step sof3d_cfuns.c:624-661
  void step2(bool forw1, bool forw2, R* trace1, R* trace2, const R* pp1, const R* pp2,
             R* trace) {
    regularization();
    w1.define(forw1, pp1, diag.data(), offd);
    w2.define(forw2, pp2, diag.data(), offd);
    slv.define(diag.data(), offd);
    R t0 = (R)(0.5 * (trace1[0] + trace2[0]));
    R t1 = (R)(0.5 * (trace1[1] + trace2[1]));
    R t2 = (R)(0.5 * (trace1[n1 - 2] + trace2[n1 - 2]));
    R t3 = (R)(0.5 * (trace1[n1 - 1] + trace2[n1 - 1]));
    w1.set(false, trace1, offd[0].data(), trace);
    w2.set(false, trace2, offd[1].data(), trace);
    for (int i1 = 0; i1 < n1; i1++) trace[i1] = offd[0][i1] + offd[1][i1];
    trace[0] += eps2 * t0;
    trace[1] += eps2 * t1;
    trace[n1 - 2] += eps2 * t2;
    trace[n1 - 1] += eps2 * t3;
    slv.solve(trace);
  }
};

// ---------------------------------------------------------------------------
// 2-D plane-wave spray, pwspray_lop sof_cfuns.c:948-1033.  u: [n2][ns2][n1].
// ---------------------------------------------------------------------------
template <class R>
static void pwspray2(Predict<R>& pr, bool adj, int n1, int n2, int ns, const R* pp, R* u1,
                     R* u) {
  int ns2 = 2 * ns + 1;
  std::vector<R> trace(n1);
  long n = (long)n1 * n2;
  if (adj) {  // add=true in the only caller (pwsmooth_lop adjoint)
    for (int i = 0; i < n2; i++) {
      for (int i1 = 0; i1 < n1; i1++) trace[i1] = 0;
      for (int is = ns - 1; is >= 0; is--) {
        int ip = i + is + 1;
        if (ip >= n2) continue;
        long j = (long)ip * ns2 + ns + is + 1;
        for (int i1 = 0; i1 < n1; i1++) trace[i1] += u[j * n1 + i1];
        pr.step(true, true, trace.data(), pp + (long)(ip - 1) * n1);
      }
      for (int i1 = 0; i1 < n1; i1++) {
        u1[(long)i * n1 + i1] += trace[i1];
        trace[i1] = 0;
      }
      for (int is = ns - 1; is >= 0; is--) {
        int ip = i - is - 1;
        if (ip < 0) continue;
        long j = (long)ip * ns2 + ns - is - 1;
        for (int i1 = 0; i1 < n1; i1++) trace[i1] += u[j * n1 + i1];
        pr.step(true, false, trace.data(), pp + (long)ip * n1);
      }
      for (int i1 = 0; i1 < n1; i1++) {
        u1[(long)i * n1 + i1] += trace[i1];
        trace[i1] = u[((long)i * ns2 + ns) * n1 + i1];
        u1[(long)i * n1 + i1] += trace[i1];
      }
    }
    return;
  }
  for (long i = 0; i < n * ns2; i++) u[i] = 0;
  for (int i = 0; i < n2; i++) {
    for (int i1 = 0; i1 < n1; i1++) {
      trace[i1] = u1[(long)i * n1 + i1];
      u[((long)i * ns2 + ns) * n1 + i1] += trace[i1];
    }
    for (int is = 0; is < ns; is++) {
      int ip = i - is - 1;
      if (ip < 0) break;
      long j = (long)ip * ns2 + ns - is - 1;
      pr.step(false, false, trace.data(), pp + (long)ip * n1);
      for (int i1 = 0; i1 < n1; i1++) u[j * n1 + i1] += trace[i1];
    }
    for (int i1 = 0; i1 < n1; i1++) trace[i1] = u1[(long)i * n1 + i1];
    for (int is = 0; is < ns; is++) {
      int ip = i + is + 1;
      if (ip >= n2) break;
      long j = (long)ip * ns2 + ns + is + 1;
      pr.step(false, true, trace.data(), pp + (long)(ip - 1) * n1);
      for (int i1 = 0; i1 < n1; i1++) u[j * n1 + i1] += trace[i1];
    }
  }
}

// csomean2d sof_cfuns.c:1433-1531 with pwsmooth_* :1036-1122: triangle-
// weighted, normalised spray mean (quirk Q4), slice by slice over n3.
template <class R>
static int somean2d(const R* din, const R* dip, R* dout, int n1, int n2, int n3, int ns,
                    int order, R eps, int adj) {
  if (n1 < 4 || n2 < 1 || n3 < 1 || ns < 0 || order < 1 || order > 8) return ORC_EINVAL;
  int ns2 = 2 * ns + 1;
  long n12 = (long)n1 * n2;
  Predict<R> pr;
  pr.init(n1, eps * eps, order, false);  // pwspray_init :915-932
  std::vector<R> u(n12 * ns2), w(ns2), w1(n12), t(n12);
  for (int is = 0; is < ns2; is++) w[is] = (R)(ns + 1 - std::abs(is - ns));
  for (int i3 = 0; i3 < n3; i3++) {
    const R* pp = dip + i3 * n12;
    // pwsmooth_set :1102-1122
    for (long i = 0; i < n12; i++) w1[i] = 1;
    pwspray2(pr, false, n1, n2, ns, pp, w1.data(), u.data());
    for (long i = 0; i < n12; i++) t[i] = 0;
    for (int i2 = 0; i2 < n2; i2++)
      for (int i1 = 0; i1 < n1; i1++) {
        R ws = w1[(long)i2 * n1 + i1];
        for (int is = 0; is < ns2; is++)
          t[(long)i2 * n1 + i1] += u[((long)i2 * ns2 + is) * n1 + i1] * w[is] * ws;
      }
    for (long i = 0; i < n12; i++) w1[i] = (t[i] != (R)0) ? (R)(1.0 / t[i]) : (R)0;
    // pwsmooth_lop :1064-1100
    const R* x = din + i3 * n12;
    R* y = dout + i3 * n12;
    if (adj) {
      for (int i2 = 0; i2 < n2; i2++)
        for (int i1 = 0; i1 < n1; i1++) {
          R ws = w1[(long)i2 * n1 + i1];
          for (int is = 0; is < ns2; is++)
            u[((long)i2 * ns2 + is) * n1 + i1] = x[(long)i2 * n1 + i1] * w[is] * ws;
        }
      for (long i = 0; i < n12; i++) y[i] = 0;
      pwspray2(pr, true, n1, n2, ns, pp, y, u.data());
    } else {
      pwspray2(pr, false, n1, n2, ns, pp, const_cast<R*>(x), u.data());
      for (long i = 0; i < n12; i++) y[i] = 0;
      for (int i2 = 0; i2 < n2; i2++)
        for (int i1 = 0; i1 < n1; i1++) {
          R ws = w1[(long)i2 * n1 + i1];
          for (int is = 0; is < ns2; is++)
            y[(long)i2 * n1 + i1] += u[((long)i2 * ns2 + is) * n1 + i1] * w[is] * ws;
        }
    }
  }
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// Sparse-data interpolation, csint2d soint2d_cfuns.c:2421-2523: shaping-
// regularised CG (ps_conjgrad :888-1012 with prec = NULL and a given initial
// model) whose operator is the known-sample mask (ps_mask_lop :145-157) and
// whose shaping is the normalised plane-wave smoothing (pwsmooth_* :2160-
// 2240, the operator csomean2d applies, on pwspray :2038-2150).
// ---------------------------------------------------------------------------
template <class R>
struct PwSmooth2 {
  int n1 = 0, n2 = 0, ns = 0, ns2 = 0;
  long n12 = 0;
  Predict<R> pr;
  std::vector<R> u, w, w1, t;
  const R* pp = nullptr;
  void init(int nr, int m1, int m2, int order, R eps) {
    n1 = m1;
    n2 = m2;
    ns = nr;
    ns2 = 2 * ns + 1;
    n12 = (long)n1 * n2;
    pr.init(n1, eps * eps, order, false);
    u.assign(n12 * ns2, 0);
    w.resize(ns2);
    for (int is = 0; is < ns2; is++) w[is] = (R)(ns + 1 - std::abs(is - ns));
    w1.assign(n12, 0);
    t.assign(n12, 0);
  }
  // pwsmooth_lop: smooth (+)= S trace, or trace (+)= S' smooth
  void lop(bool adj, bool add, R* trace, R* smooth) {
    if (!add) {
      R* z = adj ? trace : smooth;
      for (long i = 0; i < n12; i++) z[i] = 0;
    }
    if (adj) {
      for (int i2 = 0; i2 < n2; i2++)
        for (int i1 = 0; i1 < n1; i1++) {
          const R ws = w1[(long)i2 * n1 + i1];
          for (int is = 0; is < ns2; is++)
            u[((long)i2 * ns2 + is) * n1 + i1] = smooth[(long)i2 * n1 + i1] * w[is] * ws;
        }
      pwspray2(pr, true, n1, n2, ns, pp, trace, u.data());
    } else {
      pwspray2(pr, false, n1, n2, ns, pp, trace, u.data());
      for (int i2 = 0; i2 < n2; i2++)
        for (int i1 = 0; i1 < n1; i1++) {
          const R ws = w1[(long)i2 * n1 + i1];
          for (int is = 0; is < ns2; is++)
            smooth[(long)i2 * n1 + i1] += u[((long)i2 * ns2 + is) * n1 + i1] * w[is] * ws;
        }
    }
  }
  // pwsmooth_set: the slope and the normalisation 1 / S 1
  void set(const R* dip) {
    pp = dip;
    for (long i = 0; i < n12; i++) w1[i] = 1;
    lop(false, false, w1.data(), t.data());
    for (long i = 0; i < n12; i++) w1[i] = (t[i] != (R)0) ? (R)(1.0 / t[i]) : (R)0;
  }
};

// ps_conjgrad with oper = the mask of `known`, shape = S, a given initial
// model p (hasp0) and x, dat the same array (csint2d passes mm for both).
template <class R, class Shape>
static void conjgrad_masked(Shape& S, const std::vector<char>& known, long n, R eps1, R tol,
                            R* p, R* x, int niter) {
  const R eps = eps1 * eps1;
  std::vector<R> r(n), sp(n), gp(n), sx(n), gx(n), sr(n), gr(n);
  for (long i = 0; i < n; i++) r[i] = -x[i];  // r = -dat before x is overwritten
  S.lop(false, false, p, x);                   // x = S p
  for (long i = 0; i < n; i++)
    if (known[i]) r[i] += x[i];                // r += M x
  double gn, gnp = 0., alpha, beta, g0 = 0., dg = 0., r0;
  r0 = dsdot(n, r.data(), r.data());
  if (r0 == 0.) return;
  for (int iter = 0; iter < niter; iter++) {
    for (long i = 0; i < n; i++) gp[i] = eps * p[i];
    for (long i = 0; i < n; i++) gx[i] = -eps * x[i];
    for (long i = 0; i < n; i++)
      if (known[i]) gx[i] += r[i];              // gx += M' r
    S.lop(true, true, gp.data(), gx.data());    // gp += S' gx
    S.lop(false, false, gp.data(), gx.data());  // gx = S gp
    for (long i = 0; i < n; i++) gr[i] = 0;
    for (long i = 0; i < n; i++)
      if (known[i]) gr[i] += gx[i];             // gr = M gx
    gn = dsdot(n, gp.data(), gp.data());
    if (iter == 0) {
      g0 = gn;
      sp = gp;
      sx = gx;
      sr = gr;
    } else {
      alpha = gn / gnp;
      dg = gn / g0;
      if (alpha < (double)tol || dg < (double)tol) break;
      const R a = (R)alpha;
      saxpy(n, a, sp.data(), gp.data());
      std::swap(sp, gp);
      saxpy(n, a, sx.data(), gx.data());
      std::swap(sx, gx);
      saxpy(n, a, sr.data(), gr.data());
      std::swap(sr, gr);
    }
    beta = dsdot(n, sr.data(), sr.data()) +
           (double)eps * (dsdot(n, sp.data(), sp.data()) - dsdot(n, sx.data(), sx.data()));
    alpha = -gn / beta;
    const R a = (R)alpha;
    saxpy(n, a, sp.data(), p);
    saxpy(n, a, sx.data(), x);
    saxpy(n, a, sr.data(), r.data());
    gnp = gn;
  }
}

template <class R>
static int sint2d(const R* din, const R* dip, const R* mask, R* dout, int n1, int n2, int niter,
                  int ns, int order, R eps) {
  if (n1 < 4 || n2 < 1 || ns < 0 || order < 1 || order > 8 || niter < 0) return ORC_EINVAL;
  const long n12 = (long)n1 * n2;
  PwSmooth2<R> S;
  S.init(ns, n1, n2, order, eps);
  std::vector<R> xx(din, din + n12);
  for (long i = 0; i < n12; i++) dout[i] = din[i];
  std::vector<char> known(n12);
  R lam = 0;
  for (long i = 0; i < n12; i++) {
    known[i] = mask[i] != (R)0;
    if (known[i]) lam += (R)1.;
  }
  lam = std::sqrt(lam / (R)n12);
  const R tol = (R)(10 * std::numeric_limits<float>::epsilon());
  S.set(dip);
  conjgrad_masked(S, known, n12, lam, tol, xx.data(), dout, niter);
  return ORC_OK;
}

// csint3d soint3d_cfuns.c:2510-2612: the same CG with the 3-D smoothing
// pwsmooth3_lop (:2157-2300): the 2-D smoothing along the inline slope on
// every (n1, n2) slice, then along the crossline slope on every (n1, n3)
// section (the cube transposed to [n2][n3][n1]); the adjoint in reverse,
// adding into the model.
template <class R>
struct PwSmooth3 {
  int n1 = 0, n2 = 0, n3 = 0, ns1 = 0, ns2 = 0, order1 = 0, order2 = 0;
  R eps = 0;
  const R* pi = nullptr;
  std::vector<R> xd, itmp, itmp2, xtmp;  // xd: crossline slope as [n2][n3][n1]
  PwSmooth2<R> S;
  void init(int r1, int r2, int m1, int m2, int m3, int o1, int o2, R e, const R* dipi,
            const R* dipx) {
    n1 = m1;
    n2 = m2;
    n3 = m3;
    ns1 = r1;
    ns2 = r2;
    order1 = o1;
    order2 = o2;
    eps = e;
    pi = dipi;
    const long n = (long)n1 * n2 * n3;
    xd.resize(n);
    itmp.assign(n, 0);
    itmp2.assign(n, 0);
    xtmp.assign(n, 0);
    for (int i3 = 0; i3 < n3; i3++)
      for (int i2 = 0; i2 < n2; i2++)
        for (int i1 = 0; i1 < n1; i1++)
          xd[i1 + (long)n1 * (i3 + (long)n3 * i2)] = dipx[i1 + (long)n1 * (i2 + (long)n2 * i3)];
  }
  long ixc(int i1, int i2, int i3) const { return i1 + (long)n1 * (i2 + (long)n2 * i3); }
  long ixt(int i1, int i2, int i3) const { return i1 + (long)n1 * (i3 + (long)n3 * i2); }
  void lop(bool adj, bool add, R* trace, R* smooth) {
    const long n = (long)n1 * n2 * n3, n12 = (long)n1 * n2, n13 = (long)n1 * n3;
    if (!add) {
      R* z = adj ? trace : smooth;
      for (long i = 0; i < n; i++) z[i] = 0;
    }
    if (adj) {
      for (int i3 = 0; i3 < n3; i3++)
        for (int i2 = 0; i2 < n2; i2++)
          for (int i1 = 0; i1 < n1; i1++) xtmp[ixt(i1, i2, i3)] = smooth[ixc(i1, i2, i3)];
      S.init(ns2, n1, n3, order2, eps);
      for (int i2 = 0; i2 < n2; i2++) {
        S.set(xd.data() + i2 * n13);
        S.lop(true, false, itmp2.data() + i2 * n13, xtmp.data() + i2 * n13);
      }
      for (int i3 = 0; i3 < n3; i3++)
        for (int i2 = 0; i2 < n2; i2++)
          for (int i1 = 0; i1 < n1; i1++) itmp[ixc(i1, i2, i3)] = itmp2[ixt(i1, i2, i3)];
      S.init(ns1, n1, n2, order1, eps);
      for (int i3 = 0; i3 < n3; i3++) {
        S.set(pi + i3 * n12);
        S.lop(true, true, trace + i3 * n12, itmp.data() + i3 * n12);
      }
    } else {
      S.init(ns1, n1, n2, order1, eps);
      for (int i3 = 0; i3 < n3; i3++) {
        S.set(pi + i3 * n12);
        S.lop(false, false, trace + i3 * n12, itmp.data() + i3 * n12);
      }
      for (int i3 = 0; i3 < n3; i3++)
        for (int i2 = 0; i2 < n2; i2++)
          for (int i1 = 0; i1 < n1; i1++) itmp2[ixt(i1, i2, i3)] = itmp[ixc(i1, i2, i3)];
      S.init(ns2, n1, n3, order2, eps);
      for (int i2 = 0; i2 < n2; i2++) {
        S.set(xd.data() + i2 * n13);
        S.lop(false, false, itmp2.data() + i2 * n13, xtmp.data() + i2 * n13);
      }
      for (int i3 = 0; i3 < n3; i3++)
        for (int i2 = 0; i2 < n2; i2++)
          for (int i1 = 0; i1 < n1; i1++) smooth[ixc(i1, i2, i3)] += xtmp[ixt(i1, i2, i3)];
    }
  }
};

template <class R>
static int sint3d(const R* din, const R* dipi, const R* dipx, const R* mask, R* dout, int n1,
                  int n2, int n3, int niter, int ns1, int ns2, int order1, int order2, R eps) {
  if (n1 < 4 || n2 < 1 || n3 < 1 || ns1 < 0 || ns2 < 0 || order1 < 1 || order1 > 8 ||
      order2 < 1 || order2 > 8 || niter < 0)
    return ORC_EINVAL;
  const long n = (long)n1 * n2 * n3;
  std::vector<R> xx(din, din + n);
  for (long i = 0; i < n; i++) dout[i] = din[i];
  std::vector<char> known(n);
  R lam = 0;
  for (long i = 0; i < n; i++) {
    known[i] = mask[i] != (R)0;
    if (known[i]) lam += (R)1.;
  }
  lam = std::sqrt(lam / (R)n);
  PwSmooth3<R> S;
  S.init(ns1, ns2, n1, n2, n3, order1, order2, eps, dipi, dipx);
  const R tol = (R)(10 * std::numeric_limits<float>::epsilon());
  conjgrad_masked(S, known, n, lam, tol, xx.data(), dout, niter);
  return ORC_OK;
}

// Plane-wave painting, cpaint2d paint_cfuns.c:1861-1940 (called by pwpaintc
// and rgt, rgt.py:4-87): the seed trace placed at trace i0 and carried
// trace by trace to both ends by the PWD prediction step (predict_step
// :1247-1274), leftwards along the slope of the trace it leaves, rightwards
// along the slope of the trace before the one it reaches.
template <class R>
static int paint2d(const R* dip, const R* seed, R* out, int n1, int n2, int order, int i0,
                   R eps) {
  if (n1 < 4 || n2 < 1 || order < 1 || order > 8 || i0 < 0 || i0 >= n2) return ORC_EINVAL;
  Predict<R> pr;
  pr.init(n1, eps * eps, order, false);
  std::vector<R> tr(seed, seed + n1);
  for (int i1 = 0; i1 < n1; i1++) out[(long)i0 * n1 + i1] = tr[i1];
  for (int i2 = i0 - 1; i2 >= 0; i2--) {
    pr.step(false, false, tr.data(), dip + (long)i2 * n1);
    for (int i1 = 0; i1 < n1; i1++) out[(long)i2 * n1 + i1] = tr[i1];
  }
  for (int i1 = 0; i1 < n1; i1++) tr[i1] = out[(long)i0 * n1 + i1];
  for (int i2 = i0 + 1; i2 < n2; i2++) {
    pr.step(false, true, tr.data(), dip + (long)(i2 - 1) * n1);
    for (int i1 = 0; i1 < n1; i1++) out[(long)i2 * n1 + i1] = tr[i1];
  }
  return ORC_OK;
}

// Radon coherence, cohc_fb coh_cfuns.c:415-545 with coh_init2 :158-179 and
// coh :181-225 (called by cohc, das.py:92).  Forward (forw 1): data[ih][it]
// += model[iv][itau] along t(itau, ih, iv) (linear itau dt + h v, parabolic
// itau dt + h^2 v / hmax^2, hyperbolic sqrt(tau^2 + (h/v)^2)); adjoint
// (forw -1): the stack num and the energy den of the data along the same
// curves and model = num^2 / (nh den + 1e-16).  Sample index floor(t/dt) + 1
// is used as the reference uses it: up to nt, which is the next trace's
// first sample (flat indexing).  On the last trace that is one past the
// data array, which the reference writes (forward; its output never shows
// it, dropped here) or reads (adjoint; an undefined value, so the model
// samples whose stack includes it are NaN here).  The parabolic type's hmax
// is the reference's file-scope static (never reset, set to the signed
// offset of the largest magnitude): the caller passes and keeps it.
static int coh_radon(const float* in, const float* v, const float* h, int typ, int nt, int nv,
                     int nh, float dt, int forw, float* out, float* hmax) {
  if (nt < 1 || nv < 1 || nh < 1 || (forw != 1 && forw != -1)) return ORC_EINVAL;
  if (typ != 1 && typ != 2 && typ != 3) typ = 1;
  if (typ == 2)
    for (int i = 0; i < nh; i++)
      if (*hmax < std::fabs((double)h[i])) *hmax = h[i];
  const long ndata = (long)nt * nh, nmod = (long)nt * nv;
  // the sample indices first, so that a refused call writes nothing
  std::vector<int> its((size_t)nt * nh * nv);
  for (int itau = 0; itau < nt; itau++)
    for (int ih = 0; ih < nh; ih++)
      for (int iv = 0; iv < nv; iv++) {
        float t = 0.f;
        if (typ == 1) t = (float)itau * dt + h[ih] * v[iv];
        if (typ == 2) t = (float)itau * dt + h[ih] * h[ih] * v[iv] / *hmax / *hmax;
        if (typ == 3) {
          const float tau = (float)itau * dt, hv = h[ih] / v[iv];
          t = std::sqrt(tau * tau + hv * hv);
        }
        const float fl = std::floor(t / dt) + 1;
        if (!(std::fabs(fl) < 2.0e9f)) return ORC_EINVAL;
        its[((size_t)itau * nh + ih) * nv + iv] = (int)fl;
      }
  if (forw == 1) {
    for (long i = 0; i < ndata; i++) out[i] = 0.f;
    for (int itau = 0; itau < nt; itau++)
      for (int ih = 0; ih < nh; ih++)
        for (int iv = 0; iv < nv; iv++) {
          const int it = its[((size_t)itau * nh + ih) * nv + iv];
          const long id = (long)ih * nt + it;
          if (it <= nt && it + 1 > 0 && id < ndata) out[id] += in[(long)iv * nt + itau];
        }
    return ORC_OK;
  }
  std::vector<float> num(nmod, 0.f), den(nmod, 0.f);
  std::vector<char> undefined(nmod, 0);
  for (int itau = 0; itau < nt; itau++)
    for (int ih = 0; ih < nh; ih++)
      for (int iv = 0; iv < nv; iv++) {
        const int it = its[((size_t)itau * nh + ih) * nv + iv];
        if (it <= nt && it + 1 > 0) {
          const long id = (long)ih * nt + it, m = (long)iv * nt + itau;
          if (id >= ndata) {
            undefined[m] = 1;
            continue;
          }
          const float y = in[id];
          num[m] = num[m] + y;
          den[m] = den[m] + y * y;
        }
      }
  for (int itau = 0; itau < nt; itau++)
    for (int iv = 0; iv < nv; iv++) {
      const long m = (long)iv * nt + itau;
      out[m] = undefined[m] ? std::numeric_limits<float>::quiet_NaN()
                            : (float)((double)(num[m] * num[m]) /
                                      ((double)((float)nh * den[m]) + 0.0000000000000001));
    }
  return ORC_OK;
}

// sf_quantile sof_cfuns.c:1137-1163 (Hoare-style selection, a is changed)
template <class R>
static R quantile(int q, int n, R* a) {
  R *i, *j, ak, *low, *hi, buf, *k;
  low = a;
  hi = a + n - 1;
  k = a + q;
  while (low < hi) {
    ak = *k;
    i = low;
    j = hi;
    do {
      while (*i < ak) i++;
      while (*j > ak) j--;
      if (i <= j) {
        buf = *i;
        *i++ = *j;
        *j-- = buf;
      }
    } while (i <= j);
    if (j < k) low = i;
    if (k < i) hi = j;
  }
  return *k;
}

// Median filter along the spray axis of one trace's spray panel tt[np][n1]
// (mf_init axis=2 ifbound=1 :1170-1188, boundary :1218-1292, mf :1294-1332,
// svmf_init/svmf :1190-1216/:1334-1431).  Only row `row` of the result is
// produced (quirk Q7: the reference filters every row but outputs one).
template <class R>
struct SprayMedian {
  int n1, np, nmf, option;
  std::vector<R> ext, tmp, trace2;
  int m;  // nfilter2 of the first pass
  void init(int n1_, int np_, int nmf_, int option_) {
    n1 = n1_; np = np_; nmf = nmf_; option = option_;
    int nfilter = (option == 1) ? nmf : nmf + 2;
    m = (nfilter - 1) / 2;
    // One row more than boundary() fills: svmf's first pass reads one row
    // past the padded panel for its last row (sof_cfuns.c:1366-1376, an
    // out-of-bounds read in the reference); here that row is one more
    // replica of the last trace, as the padding rows are.
    ext.assign((long)n1 * (np + 2 * m + 1), 0);
    tmp.assign(nfilter + 8, 0);
    trace2.assign((long)n1 * np, 0);
  }
  void extend(const R* tt) {  // boundary(), axis 2, edge replication
    for (int i = 0; i < m; i++)
      for (int j = 0; j < n1; j++) ext[(long)n1 * i + j] = tt[j];
    for (int i = 0; i < np; i++)
      for (int j = 0; j < n1; j++) ext[(long)n1 * (i + m) + j] = tt[(long)n1 * i + j];
    for (int i = 0; i < m + 1; i++)
      for (int j = 0; j < n1; j++) ext[(long)n1 * (i + np + m) + j] = tt[(long)n1 * (np - 1) + j];
  }
  // out[n1] = row `row` of the filtered panel
  void apply(const R* tt, int row, R* out) {
    extend(tt);
    if (option == 1) {
      for (int j = 0; j < n1; j++) {
        for (int k = 0; k < nmf; k++) tmp[k] = ext[(long)n1 * (row + k) + j];
        out[j] = quantile(m, nmf, tmp.data());
      }
      return;
    }
    // svmf: first pass over every row with window nmf+2 (l1=2), offset m-m2
    int nfilter = nmf + 2;
    int m2 = (nmf - 1) / 2;
    for (int i = 0; i < np; i++)
      for (int j = 0; j < n1; j++) {
        for (int k = 0; k < nfilter; k++) tmp[k] = ext[(long)n1 * (m + i + k - m2) + j];
        trace2[(long)n1 * i + j] = quantile(m, nfilter, tmp.data());
      }
    R sum = 0;
    for (long i = 0; i < (long)n1 * np; i++) sum = (R)(sum + std::fabs((double)trace2[i]));
    R avg = sum / (R)(n1 * np);
    for (int j = 0; j < n1; j++) {
      long i = (long)row * n1 + j;
      R a = std::fabs(tt[i]);
      int wl;
      if (a < avg)
        wl = (a < avg / 2) ? nmf + 2 : nmf + 0;
      else
        wl = (a > avg * 2) ? nmf - 4 : nmf - 2;
      int mm2 = (wl - 1) / 2;
      for (int k = 0; k < wl; k++) tmp[k] = ext[(long)n1 * (row + m + k - mm2) + j];
      out[j] = quantile(mm2, wl, tmp.data());
    }
  }
};

// csomf2d sof_cfuns.c:1534-1678
template <class R>
static int somf2d(const R* din, const R* dip, R* dout, int n1, int n2, int n3, int ns, int nmf,
                  int option, int order, R eps) {
  if (n1 < 4 || n2 < 1 || n3 < 1 || ns < 0 || order < 1 || order > 8 || nmf < 1) return ORC_EINVAL;
  if (option != 1 && nmf < 5) return ORC_EINVAL;  // svmf windows of nmf-4 must be >= 1
  int ns2 = 2 * ns + 1;
  long n12 = (long)n1 * n2;
  Predict<R> pr;
  pr.init(n1, eps * eps, order, false);
  std::vector<R> u(n12 * ns2);
  SprayMedian<R> med;
  med.init(n1, ns2, nmf, option);
  for (int i3 = 0; i3 < n3; i3++) {
    pwspray2(pr, false, n1, n2, ns, dip + i3 * n12, const_cast<R*>(din + i3 * n12), u.data());
    for (int i = 0; i < n2; i++)
      med.apply(u.data() + (long)i * ns2 * n1, (ns2 - 1) / 2, dout + i3 * n12 + (long)i * n1);
  }
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// 3-D spray over the (2r1+1)x(2r2+1) offset grid, csomean3d
// sof3d_cfuns.c:1355-1551 with update_init/get_update :980-1056.
// ---------------------------------------------------------------------------
struct Update {
  int un1, un2;
  std::vector<float> t0;
  std::vector<int> visit;
  void init(int m1, int m2, const std::vector<float>& t) {
    un1 = m1; un2 = m2; t0 = t;
    visit.resize((size_t)m1 * m2);
    for (int i = 0; i < m1 * m2; i++) visit[i] = i;
    // Any order sorted by t gives the same spray: a predecessor always has a
    // strictly smaller t.
    std::stable_sort(visit.begin(), visit.end(), [&](int a, int b) { return t0[a] < t0[b]; });
  }
  int get(int i, bool* up1, bool* up2, int* j) const {
    *j = visit[i];
    float t1 = t0[*j];
    int i1 = *j % un1, i2 = *j / un1;
    int update = 0;
    if (un1 > 1) {
      int a1 = *j - 1, b1 = *j + 1;
      *up1 = (i1 && (i1 == un1 - 1 || !(t0[a1] > t0[b1])));
      int c1 = *up1 ? a1 : b1;
      if (t1 > t0[c1]) update |= 1;
    }
    if (un2 > 1) {
      int a2 = *j - un1, b2 = *j + un1;
      *up2 = (i2 && (i2 == un2 - 1 || !(t0[a2] > t0[b2])));
      int c2 = *up2 ? a2 : b2;
      if (t1 > t0[c2]) update |= 2;
    }
    return update;
  }
};

// Sprays every trace over the offset grid: u[n23][np][n1].
template <class R>
static void pwspray3(int n1, int n2, int n3, int ns2, int ns3, int order, const R* din,
                     const R* p1, const R* p2, R* u) {
  int np2 = 2 * ns2 + 1, np3 = 2 * ns3 + 1, np = np2 * np3;
  long n23 = (long)n2 * n3;
  std::vector<float> cost((size_t)np);
  for (int i3 = 0; i3 < np3; i3++)
    for (int i2 = 0; i2 < np2; i2++) cost[i3 * np2 + i2] = hypotf((float)(i2 - ns2), (float)(i3 - ns3));
  R eps = (R)0.01f;  // quirk Q3: csomean3d/csomf3d force eps=0.01
  Predict<R> pr;
  pr.init(n1, eps * eps, order, true);
  Update up;
  up.init(np2, np3, cost);
  for (long i = 0; i < n23 * np * n1; i++) u[i] = 0;
  auto U = [&](long tr, int slot) { return u + (tr * np + slot) * (long)n1; };
  bool up2 = false, up3 = false;
  for (long i = 0; i < n23; i++) {
    for (int j = 0; j < n1; j++) U(i, ns3 * np2 + ns2)[j] = din[i * n1 + j];
    int i2 = (int)(i % n2), i3 = (int)(i / n2);
    for (int ip = 0; ip < np; ip++) {
      int jp;
      int update = up.get(ip, &up2, &up3, &jp);
      int k2 = jp % np2, k3 = jp / np2;
      long j2 = i2 + k2 - ns2, j3 = i3 + k3 - ns3;
      if (j2 < 0 || j2 >= n2 || j3 < 0 || j3 >= n3) continue;
      long j = j2 + j3 * n2;
      R* trace = U(j, jp);
      const R *q2 = nullptr, *q3 = nullptr;
      if (update & 1) {
        if (up2) {
          if (j2 == 0) continue;
          j2 = j - 1; q2 = p1 + j2 * n1; k2 = jp - 1;
        } else {
          if (j2 == n2 - 1) continue;
          j2 = j + 1; q2 = p1 + j * n1; k2 = jp + 1;
        }
      }
      if (update & 2) {
        if (up3) {
          if (j3 == 0) continue;
          j3 = j - n2; q3 = p2 + j3 * n1; k3 = jp - np2;
        } else {
          if (j3 == n3 - 1) continue;
          j3 = j + n2; q3 = p2 + j * n1; k3 = jp + np2;
        }
      }
      switch (update) {
        case 1: pr.step1(up2, U(j2, k2), q2, trace); break;
        case 2: pr.step1(up3, U(j3, k3), q3, trace); break;
        case 3: pr.step2(up2, up3, U(j2, k2), U(j3, k3), q2, q3, trace); break;
        default: break;
      }
    }
  }
}

template <class R>
static int somean3d(const R* din, const R* p1, const R* p2, R* dout, int n1, int n2, int n3,
                    int r1, int r2, int order) {
  if (n1 < 4 || n2 < 1 || n3 < 1 || r1 < 0 || r2 < 0 || order < 1 || order > 8) return ORC_EINVAL;
  int np = (2 * r1 + 1) * (2 * r2 + 1);
  long n23 = (long)n2 * n3;
  std::vector<R> u(n23 * np * n1);
  pwspray3(n1, n2, n3, r1, r2, order, din, p1, p2, u.data());
  for (long i = 0; i < n23; i++)
    for (int k = 0; k < n1; k++) {
      R sum = 0;
      for (int j = 0; j < np; j++) sum = sum + u[(i * np + j) * n1 + k];
      sum = sum / (R)np;
      dout[i * n1 + k] = sum;
    }
  return ORC_OK;
}

// csomf3d sof3d_cfuns.c:1554-1753: median over rmf raster-ordered slots
// centred on slot (np-1)/2 (quirk Q5), or svmf.
template <class R>
static int somf3d(const R* din, const R* p1, const R* p2, R* dout, int n1, int n2, int n3,
                  int r1, int r2, int nmf, int option, int order) {
  if (n1 < 4 || n2 < 1 || n3 < 1 || r1 < 0 || r2 < 0 || order < 1 || order > 8 || nmf < 1)
    return ORC_EINVAL;
  if (option != 1 && nmf < 5) return ORC_EINVAL;
  int np = (2 * r1 + 1) * (2 * r2 + 1);
  long n23 = (long)n2 * n3;
  std::vector<R> u(n23 * np * n1);
  pwspray3(n1, n2, n3, r1, r2, order, din, p1, p2, u.data());
  SprayMedian<R> med;
  med.init(n1, np, nmf, option);
  for (long i = 0; i < n23; i++) med.apply(u.data() + i * np * n1, (np - 1) / 2, dout + i * n1);
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// soint3d: PWD-regularised interpolation, csoint3d soint3d_cfuns.c:2405-2507.
// ---------------------------------------------------------------------------
struct MT19937 {  // MT19937 (Matsumoto & Nishimura), soint3d_cfuns.c:2303-2373
  uint32_t mt[624];
  int mti = 625;
  void seed(uint32_t s) {
    mt[0] = s;
    for (mti = 1; mti < 624; mti++)
      mt[mti] = 1812433253u * (mt[mti - 1] ^ (mt[mti - 1] >> 30)) + (uint32_t)mti;
  }
  uint32_t next() {
    static const uint32_t mag01[2] = {0u, 0x9908b0dfu};
    uint32_t y;
    if (mti >= 624) {
      if (mti == 625) seed(5489u);
      int kk;
      for (kk = 0; kk < 624 - 397; kk++) {
        y = (mt[kk] & 0x80000000u) | (mt[kk + 1] & 0x7fffffffu);
        mt[kk] = mt[kk + 397] ^ (y >> 1) ^ mag01[y & 1u];
      }
      for (; kk < 623; kk++) {
        y = (mt[kk] & 0x80000000u) | (mt[kk + 1] & 0x7fffffffu);
        mt[kk] = mt[kk + (397 - 624)] ^ (y >> 1) ^ mag01[y & 1u];
      }
      y = (mt[623] & 0x80000000u) | (mt[0] & 0x7fffffffu);
      mt[623] = mt[396] ^ (y >> 1) ^ mag01[y & 1u];
      mti = 0;
    }
    y = mt[mti++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
  }
  double real1() { return next() * (1.0 / 4294967295.0); }
};

// Box-Muller pair generator, ps_randn_one_bm :2378-2400 (second value of a
// pair first).  The pair state starts fresh per call: every call draws an
// even count (2n), so the reference's process-wide state is also fresh.
struct RandN {
  MT19937 g;
  bool iset = true;
  float vset = 0;
  float next() {
    if (iset) {
      double x1, x2;
      do { x1 = g.real1(); } while (x1 == 0.0);
      x2 = g.real1();
      double z1 = std::sqrt(-2.0 * std::log(x1));
      double z2 = 2.0 * 3.14159265358979323846264338328 * x2;
      double y1 = z1 * std::cos(z2), y2 = z1 * std::sin(z2);
      iset = false;
      vset = (float)y1;
      return (float)y2;
    }
    iset = true;
    return vset;
  }
};

// allpass3_lop soint3d_cfuns.c:625-730: [n] -> [2n] stacked inline and
// crossline PWD residual, and its adjoint.
template <class R>
struct Allpass3 {
  int nx, ny, nz, nw, nj1, nj2;
  bool drift;
  const R *pp, *qq;
  ApFilter<R> af;
  static int nint(R x) { return (int)((x) > 0.0 ? (x) + 0.5 : (x)-0.5); }
  void lop(bool adj, bool add, long n1, R* xx, R* yy) const {
    if (!add) {
      if (adj) for (long i = 0; i < n1; i++) xx[i] = 0;
      else for (long i = 0; i < 2 * n1; i++) yy[i] = 0;
    }
    R flt[17];
    for (int part = 0; part < 2; part++) {
      const R* p = part == 0 ? pp : qq;
      int nj = part == 0 ? nj1 : nj2;
      long st = part == 0 ? nx : (long)nx * ny;
      int iy1 = part == 0 ? ny - 1 : ny, iz1 = part == 0 ? nz : nz - 1;
      R* y = yy + (part == 0 ? 0 : n1);
      for (int iz = 0; iz < iz1; iz++)
        for (int iy = 0; iy < iy1; iy++)
          for (int ix = nw * nj; ix < nx - nw * nj; ix++) {
            long i = ix + (long)nx * (iy + (long)ny * iz);
            int id = 0;
            R pi = p[i];
            if (drift) {
              id = nint(p[i]);
              if (ix - nw * nj - id < 0 || ix + nw * nj - id >= nx) continue;
              pi = p[i] - (R)id;
            }
            af.pass(pi, flt);
            for (int iw = 0; iw <= 2 * nw; iw++) {
              int is = (iw - nw) * nj;
              if (adj) {
                xx[i + st + is] += y[i] * flt[iw];
                xx[i - is - id] -= y[i] * flt[iw];
              } else {
                y[i] += (xx[i + st + is] - xx[i - is - id]) * flt[iw];
              }
            }
          }
    }
  }
};

// ps_solver (:894-1175) restricted to the csoint3d call (known mask, x0) with
// ps_cgstep (:826-877).
template <class R>
static void solver_known(const Allpass3<R>& L, long nx, R* x, const R* dat, int niter,
                         const uint8_t* known) {
  long ny = 2 * nx;
  std::vector<R> g(nx), rr(ny), gg(ny), S(nx), Ss(ny);
  for (long i = 0; i < ny; i++) rr[i] = -dat[i];
  L.lop(false, true, nx, x, rr.data());
  R dpr0 = snrm2(ny, rr.data()), dpg0 = 1, dpr, dpg;
  const R TOL = (R)1.e-12f, EPS = (R)1.e-12f;
  bool forget = true;  // the first ps_cgstep call of a run restarts
  for (int iter = 0; iter < niter; iter++) {
    L.lop(true, false, nx, g.data(), rr.data());
    for (long i = 0; i < nx; i++)
      if (known[i]) g[i] = 0;
    L.lop(false, false, nx, g.data(), gg.data());
    if (iter == 0) {
      dpg0 = snrm2(nx, g.data());
      dpr = 1;
      dpg = 1;
    } else {
      dpr = snrm2(ny, rr.data()) / dpr0;
      dpg = snrm2(nx, g.data()) / dpg0;
    }
    if (dpr < TOL || dpg < TOL) break;
    // ps_cgstep
    double alfa, beta;
    bool skip = false;
    if (forget) {
      for (long i = 0; i < nx; i++) S[i] = 0;
      for (long i = 0; i < ny; i++) Ss[i] = 0;
      beta = 0.0;
      alfa = dsdot(ny, gg.data(), gg.data());
      if (alfa <= 0.) skip = true;
      else alfa = -dsdot(ny, gg.data(), rr.data()) / alfa;
    } else {
      double gdg = dsdot(ny, gg.data(), gg.data());
      double sds = dsdot(ny, Ss.data(), Ss.data());
      double gds = dsdot(ny, gg.data(), Ss.data());
      if (gdg == 0. || sds == 0.) {
        skip = true;
        alfa = beta = 0;
      } else {
        double determ = 1.0 - (gds / gdg) * (gds / sds);
        if (determ > (double)EPS) determ *= gdg * sds;
        else determ = gdg * sds * (double)EPS;
        double gdr = -dsdot(ny, gg.data(), rr.data());
        double sdr = -dsdot(ny, Ss.data(), rr.data());
        alfa = (sds * gdr - gds * sdr) / determ;
        beta = (-gds * gdr + gdg * sdr) / determ;
      }
    }
    forget = false;
    if (skip) continue;
    R b = (R)beta, a = (R)alfa;
    for (long i = 0; i < nx; i++) S[i] *= b;
    saxpy(nx, a, g.data(), S.data());
    for (long i = 0; i < ny; i++) Ss[i] *= b;
    saxpy(ny, a, gg.data(), Ss.data());
    for (long i = 0; i < nx; i++) x[i] += S[i];
    for (long i = 0; i < ny; i++) rr[i] += Ss[i];
  }
}

template <class R>
static int soint3d(const R* din, const R* mask, const R* pp, const R* qq, R* dout, int n1,
                   int n2, int n3, int nw, int nj1, int nj2, int niter, int drift, int seed,
                   int hasmask, R var) {
  if (n1 < 1 || n2 < 1 || n3 < 1 || nw < 1 || nw > 8 || nj1 < 1 || nj2 < 1 || niter < 0)
    return ORC_EINVAL;
  long n = (long)n1 * n2 * n3;
  R a = (R)std::sqrt((double)var);
  if (sizeof(R) == 4) a = (R)sqrtf((float)var);
  RandN rn;
  rn.g.seed((uint32_t)seed);
  std::vector<uint8_t> known(n);
  for (long i = 0; i < n; i++) known[i] = hasmask == 1 ? (mask[i] != (R)0) : (din[i] != (R)0);
  std::vector<R> dd(2 * n);
  for (long i = 0; i < 2 * n; i++) dd[i] = a * (R)rn.next();
  for (long i = 0; i < n; i++) dout[i] = din[i];
  Allpass3<R> L;
  L.nx = n1; L.ny = n2; L.nz = n3; L.nw = nw; L.nj1 = nj1; L.nj2 = nj2;
  L.drift = drift != 0; L.pp = pp; L.qq = qq;
  L.af.init(nw);
  solver_known(L, n, dout, dd.data(), niter, known.data());
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// Preconditioned 2-D interpolation, the prec = 1 branches of csoint2d
// (soint2d_cfuns.c:2354-2398): ps_solver_prec (:1704-2034) with ps_mask_lop
// (:145-159) as the operator, ps_cgstep (:493-544) as the step and
// predict_lop (:1537-1571) or predict2_lop (:1597-1616) as the
// preconditioner, x = P p, eps = 0, no weights, no x0.
// ---------------------------------------------------------------------------

// predict_lop: trace-by-trace integration along the slopes.  Forward:
// tt += xx[i2], yy[i2] += tt, tt = predict_step(tt; dip[i2]) for ascending
// i2; the adjoint runs the steps backwards.  forw = true throughout.
template <class R>
static void predict_lop(Predict<R>& pr, bool adj, bool add, int n1, int n2, const R* dip, R* xx,
                        R* yy) {
  const long n = (long)n1 * n2;
  if (!add) std::fill(adj ? xx : yy, (adj ? xx : yy) + n, (R)0);
  std::vector<R> tt(n1, (R)0);
  if (adj) {
    for (int i2 = n2 - 1; i2 >= 0; i2--) {
      pr.step(true, true, tt.data(), dip + (long)i2 * n1);
      for (int i1 = 0; i1 < n1; i1++) tt[i1] += yy[i1 + (long)i2 * n1];
      for (int i1 = 0; i1 < n1; i1++) xx[i1 + (long)i2 * n1] += tt[i1];
    }
  } else {
    for (int i2 = 0; i2 < n2; i2++) {
      for (int i1 = 0; i1 < n1; i1++) tt[i1] += xx[i1 + (long)i2 * n1];
      for (int i1 = 0; i1 < n1; i1++) yy[i1 + (long)i2 * n1] += tt[i1];
      pr.step(false, true, tt.data(), dip + (long)i2 * n1);
    }
  }
}

// The preconditioner: predict_lop with pp, or predict2_lop (the chain of
// the pp and qq integrations) when qq is given; tmp holds the
// intermediate of the chain.
template <class R>
static void prec_lop(Predict<R>& pr, bool adj, int n1, int n2, const R* pp, const R* qq, R* x,
                     R* y, R* tmp) {
  if (!qq) {
    predict_lop(pr, adj, false, n1, n2, pp, x, y);
  } else if (adj) {
    predict_lop(pr, true, false, n1, n2, qq, tmp, y);
    predict_lop(pr, true, false, n1, n2, pp, x, tmp);
  } else {
    predict_lop(pr, false, false, n1, n2, pp, x, tmp);
    predict_lop(pr, false, false, n1, n2, qq, tmp, y);
  }
}

// ps_solver_prec as csoint2d calls it: x and dat are the same array (mm);
// dat is read once, into rr = -dat, and x is the chain's intermediate until
// the final x = P p.  The model-space half of p beyond nprec (eps p = 0
// with eps = 0) never reaches x and is left out; its zeros do enter gg
// through the saxpy with eps = 0, kept here.
template <class R>
static void solver_prec(int n1, int n2, int nw, const R* pp, const R* qq, const uint8_t* known,
                        R* x, int niter) {
  const long n = (long)n1 * n2;
  Predict<R> pr;
  pr.init(n1, (R)0.0001f, nw, false);  // predict_init(n1, n2, 0.0001, nw, 1, false)
  std::vector<R> p(n, (R)0), g(n), rr(n), gg(n), S(n, (R)0), Ss(n, (R)0), tmp(n);
  for (long i = 0; i < n; i++) rr[i] = -x[i];
  double dprr, dpgm, dprr0 = 1., dpgm0 = 1.;
  const double TOL = (double)1.e-12f, EPS = (double)1.e-12f;
  bool forget = true;  // ps_cgstep's first call restarts
  for (int iter = 0; iter < niter; iter++) {
    // g = P' M rr
    for (long i = 0; i < n; i++) {
      x[i] = 0;
      if (known[i]) x[i] += rr[i];
    }
    prec_lop(pr, true, n1, n2, pp, qq, g.data(), x, tmp.data());
    // gg = M P g + eps g[nprec:] with g[nprec:] = eps rr
    prec_lop(pr, false, n1, n2, pp, qq, g.data(), x, tmp.data());
    for (long i = 0; i < n; i++) {
      gg[i] = 0;
      if (known[i]) gg[i] += x[i];
    }
    for (long i = 0; i < n; i++) gg[i] += (R)0.f * (R)(0. * rr[i]);
    if (iter == 0) {
      dprr0 = snrm2(n, rr.data());
      dpgm0 = snrm2(n, g.data());
      dprr = 1.;
      dpgm = 1.;
    } else {
      dprr = snrm2(n, rr.data()) / dprr0;
      dpgm = snrm2(n, g.data()) / dpgm0;
    }
    if (dprr < TOL || dpgm < TOL) {
      prec_lop(pr, false, n1, n2, pp, qq, p.data(), x, tmp.data());
      return;
    }
    // ps_cgstep(forget, nprec + ny, ny, p, g, rr, gg)
    double alfa = 0, beta = 0;
    bool skip = false;
    if (forget) {
      std::fill(S.begin(), S.end(), (R)0);
      std::fill(Ss.begin(), Ss.end(), (R)0);
      alfa = dsdot(n, gg.data(), gg.data());
      if (alfa <= 0.) skip = true;
      else alfa = -dsdot(n, gg.data(), rr.data()) / alfa;
    } else {
      double gdg = dsdot(n, gg.data(), gg.data());
      double sds = dsdot(n, Ss.data(), Ss.data());
      double gds = dsdot(n, gg.data(), Ss.data());
      if (gdg == 0. || sds == 0.) {
        skip = true;
      } else {
        double determ = 1.0 - (gds / gdg) * (gds / sds);
        if (determ > EPS) determ *= gdg * sds;
        else determ = gdg * sds * EPS;
        double gdr = -dsdot(n, gg.data(), rr.data());
        double sdr = -dsdot(n, Ss.data(), rr.data());
        alfa = (sds * gdr - gds * sdr) / determ;
        beta = (-gds * gdr + gdg * sdr) / determ;
      }
    }
    forget = false;
    if (!skip) {
      const R b = (R)beta, a = (R)alfa;
      for (long i = 0; i < n; i++) S[i] *= b;
      saxpy(n, a, g.data(), S.data());
      for (long i = 0; i < n; i++) Ss[i] *= b;
      saxpy(n, a, gg.data(), Ss.data());
      for (long i = 0; i < n; i++) p[i] += S[i];
      for (long i = 0; i < n; i++) rr[i] += Ss[i];
    }
    if (iter == niter - 1) prec_lop(pr, false, n1, n2, pp, qq, p.data(), x, tmp.data());
  }
}

// csoint2d with prec = 1: dout = din interpolated; known = (mask != 0)
// when hasmask == 1, else (din != 0); qq = nullptr for one plane.
template <class R>
static int soint2d_prec(const R* din, const R* mask, const R* pp, const R* qq, R* dout, int n1,
                        int n2, int nw, int niter, int hasmask) {
  if (n1 < 2 || n2 < 1 || nw < 1 || nw > 8 || niter < 0) return ORC_EINVAL;
  const long n = (long)n1 * n2;
  std::vector<uint8_t> known(n);
  for (long i = 0; i < n; i++) known[i] = hasmask == 1 ? (mask[i] != (R)0) : (din[i] != (R)0);
  for (long i = 0; i < n; i++) dout[i] = din[i];
  solver_prec(n1, n2, nw, pp, qq, known.data(), dout, niter);
  return ORC_OK;
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C ABI of the oracle (f32 = reference arithmetic, f64 = FP64 oracle).
// ---------------------------------------------------------------------------
namespace {
// Every entry point runs in the default floating-point environment (IEEE
// denormals, round to nearest), whatever libraries loaded into the process
// have set: some set flush-to-zero at load time, which the reference does
// not run with.
struct DefaultFpEnv {
  std::fenv_t saved;
  DefaultFpEnv() {
    std::fegetenv(&saved);
    std::fesetenv(FE_DFL_ENV);
  }
  ~DefaultFpEnv() { std::fesetenv(&saved); }
};
}  // namespace

// ---------------------------------------------------------------------------
// Band-pass (bp_cfuns.c:422-507 sf_butter_init / sf_butter_apply, :524-645
// cbp): Butterworth low-cut and high-cut filters of cascaded first- and
// second-order sections, run along each trace, and again from the trace's
// end for zero phase.  Coefficients follow the C expressions' types: a
// float mixed with a double constant is evaluated in double and stored as
// float; the per-sample recurrences are float, left to right.
// ---------------------------------------------------------------------------
namespace orc {

struct Butter {
  bool low = false;
  int nn = 0;
  std::vector<float> c0, c2;  // per section: gain and last feedback tap
  float mid = 0.f;             // middle feedback tap of the second-order sections
};

inline Butter butter_init(bool low, float cutoff, int nn) {
  const double pi = 3.14159265358979323846264338328;
  Butter b;
  b.low = low;
  b.nn = nn;
  b.c0.assign((nn + 1) / 2, 0.f);
  b.c2.assign((nn + 1) / 2, 0.f);
  const float arg = (float)(2. * pi * (double)cutoff);
  const float sw = sinf(arg), cw = cosf(arg);
  if (nn % 2) {  // the first-order section is the last row
    float f;
    if (low) {
      f = (float)((1. + (double)cw) / (double)sw);
      b.c0[nn / 2] = (float)(1. / (1. + (double)f));
      b.c2[nn / 2] = (float)(1. - (double)f);
    } else {
      f = (float)((double)sw / (1. + (double)cw));
      b.c0[nn / 2] = (float)(1. / ((double)f + 1.));
      b.c2[nn / 2] = (float)((double)f - 1.);
    }
  }
  const float half = (float)(0.5 * (double)arg);
  float g = low ? sinf(half) : cosf(half);
  g = g * g;
  for (int j = 0; j < nn / 2; j++) {
    const float ang = (float)(pi * (double)(2 * j + 1) / (double)(2 * nn));
    const float ss = sinf(ang) * sw;
    b.c0[j] = (float)((double)g / (1. + (double)ss));
    b.c2[j] = (float)((1. - (double)ss) / (double)g);
  }
  b.mid = (float)(-2. * (double)cw / (double)g);
  return b;
}

// The filter along x[0..nx) (back = false) or from x[nx-1] down (back =
// true: the reference's reverse, apply, reverse).
inline void butter_run(const Butter& b, int nx, float* x, bool back) {
  auto at = [&](int k) -> float& { return x[back ? nx - 1 - k : k]; };
  const int nn = b.nn;
  if (nn % 2) {
    const float c0 = b.c0[nn / 2], c2 = b.c2[nn / 2];
    float x0 = 0.f, x1, y1 = 0.f;
    for (int k = 0; k < nx; k++) {
      x1 = x0;
      x0 = at(k);
      const float s = b.low ? x0 + x1 : x0 - x1;
      y1 = (s - c2 * y1) * c0;
      at(k) = y1;
    }
  }
  for (int j = 0; j < nn / 2; j++) {
    const float c0 = b.c0[j], c2 = b.c2[j], c1 = b.mid;
    float x0 = 0.f, x1 = 0.f, x2, y1 = 0.f, y2 = 0.f;
    for (int k = 0; k < nx; k++) {
      x2 = x1;
      x1 = x0;
      x0 = at(k);
      const float tx = 2.f * x1;
      const float s = b.low ? (x0 + tx) + x2 : (x0 - tx) + x2;
      const float y0 = ((s - c1 * y1) - c2 * y2) * c0;
      y2 = y1;
      y1 = y0;
      at(k) = y0;
    }
  }
}

inline int bandpass(const float* in, float* out, int n1, long ntr, float d1, float flo,
                    float fhi, int nplo, int nphi, int phase) {
  if (n1 < 1 || ntr < 1) return ORC_EINVAL;
  const float eps = 0.0001f;
  if (!(flo < 0.f)) flo = flo * d1;  // a negative flo is kept as given
  if (!(fhi < 0.f)) fhi = fhi * d1;
  if (nplo < 1) nplo = 1;
  if (nplo > 1 && !phase) nplo /= 2;
  if (nphi < 1) nphi = 1;
  if (nphi > 1 && !phase) nphi /= 2;
  const bool lo = flo > eps, hi = (double)fhi < 0.5 - (double)eps;
  Butter blo, bhi;
  if (lo) blo = butter_init(false, flo, nplo);
  if (hi) bhi = butter_init(true, fhi, nphi);
  for (long t = 0; t < ntr; t++) {
    float* x = out + t * n1;
    if (x != in + t * n1) std::memcpy(x, in + t * n1, sizeof(float) * n1);
    if (lo) {
      butter_run(blo, n1, x, false);
      if (!phase) butter_run(blo, n1, x, true);
    }
    if (hi) {
      butter_run(bhi, n1, x, false);
      if (!phase) butter_run(bhi, n1, x, true);
    }
  }
  return 0;
}

}  // namespace orc

extern "C" {
void orc_set_store16(int mode) { orc::g_store16 = mode; }
void orc_set_cg_store16(int mode) { orc::g_cg_store16 = mode; }

int orc_dip_f32(const float* u, const float* mask, float* p, int n1, int n2, int n3, int niter,
                int liter, int order, int r1, int r2, int r3, int flags, int* ls) {
  DefaultFpEnv fpenv;
  int rect[3] = {r1, r2, r3};
  return orc::dipc<float>(u, mask, p, n1, n2, n3, niter, liter, order, rect, flags, ls);
}
int orc_dip_f64(const double* u, const double* mask, double* p, int n1, int n2, int n3,
                int niter, int liter, int order, int r1, int r2, int r3, int flags, int* ls) {
  DefaultFpEnv fpenv;
  int rect[3] = {r1, r2, r3};
  return orc::dipc<double>(u, mask, p, n1, n2, n3, niter, liter, order, rect, flags, ls);
}

int orc_pwspray2d_f32(const float* d, const float* p, float* u, int n1, int n2, int ns,
                      int order, float eps) {
  DefaultFpEnv fpenv;
  if (n1 < 4 || n2 < 1 || ns < 0 || order < 1 || order > 8) return orc::ORC_EINVAL;
  orc::Predict<float> pr;
  pr.init(n1, eps * eps, order, false);
  orc::pwspray2(pr, false, n1, n2, ns, p, const_cast<float*>(d), u);
  return 0;
}

int orc_somean2d_f32(const float* d, const float* p, float* out, int n1, int n2, int n3, int ns,
                     int order, float eps, int adj) {
  DefaultFpEnv fpenv;
  return orc::somean2d<float>(d, p, out, n1, n2, n3, ns, order, eps, adj);
}
int orc_sint2d_f32(const float* d, const float* p, const float* m, float* out, int n1, int n2,
                   int niter, int ns, int order, float eps) {
  DefaultFpEnv fpenv;
  return orc::sint2d<float>(d, p, m, out, n1, n2, niter, ns, order, eps);
}
int orc_sint3d_f32(const float* d, const float* pi, const float* px, const float* m, float* out,
                   int n1, int n2, int n3, int niter, int ns1, int ns2, int order1, int order2,
                   float eps) {
  DefaultFpEnv fpenv;
  return orc::sint3d<float>(d, pi, px, m, out, n1, n2, n3, niter, ns1, ns2, order1, order2, eps);
}
int orc_paint2d_f32(const float* dip, const float* seed, float* out, int n1, int n2, int order,
                    int i0, float eps) {
  DefaultFpEnv fpenv;
  return orc::paint2d<float>(dip, seed, out, n1, n2, order, i0, eps);
}
int orc_coh_f32(const float* in, const float* v, const float* h, int typ, int nt, int nv, int nh,
                float dt, int forw, float* out, float* hmax) {
  DefaultFpEnv fpenv;
  return orc::coh_radon(in, v, h, typ, nt, nv, nh, dt, forw, out, hmax);
}
int orc_somean2d_f64(const double* d, const double* p, double* out, int n1, int n2, int n3,
                     int ns, int order, double eps, int adj) {
  DefaultFpEnv fpenv;
  return orc::somean2d<double>(d, p, out, n1, n2, n3, ns, order, eps, adj);
}
int orc_somf2d_f32(const float* d, const float* p, float* out, int n1, int n2, int n3, int ns,
                   int nmf, int option, int order, float eps) {
  DefaultFpEnv fpenv;
  return orc::somf2d<float>(d, p, out, n1, n2, n3, ns, nmf, option, order, eps);
}
int orc_somf2d_f64(const double* d, const double* p, double* out, int n1, int n2, int n3, int ns,
                   int nmf, int option, int order, double eps) {
  DefaultFpEnv fpenv;
  return orc::somf2d<double>(d, p, out, n1, n2, n3, ns, nmf, option, order, eps);
}

int orc_pwspray3d_f32(const float* d, const float* p1, const float* p2, float* u, int n1, int n2,
                      int n3, int r1, int r2, int order) {
  DefaultFpEnv fpenv;
  if (n1 < 4 || n2 < 1 || n3 < 1 || r1 < 0 || r2 < 0 || order < 1 || order > 8)
    return orc::ORC_EINVAL;
  orc::pwspray3<float>(n1, n2, n3, r1, r2, order, d, p1, p2, u);
  return 0;
}
int orc_somean3d_f32(const float* d, const float* p1, const float* p2, float* out, int n1,
                     int n2, int n3, int r1, int r2, int order) {
  DefaultFpEnv fpenv;
  return orc::somean3d<float>(d, p1, p2, out, n1, n2, n3, r1, r2, order);
}
int orc_somean3d_f64(const double* d, const double* p1, const double* p2, double* out, int n1,
                     int n2, int n3, int r1, int r2, int order) {
  DefaultFpEnv fpenv;
  return orc::somean3d<double>(d, p1, p2, out, n1, n2, n3, r1, r2, order);
}
int orc_somf3d_f32(const float* d, const float* p1, const float* p2, float* out, int n1, int n2,
                   int n3, int r1, int r2, int nmf, int option, int order) {
  DefaultFpEnv fpenv;
  return orc::somf3d<float>(d, p1, p2, out, n1, n2, n3, r1, r2, nmf, option, order);
}
int orc_somf3d_f64(const double* d, const double* p1, const double* p2, double* out, int n1,
                   int n2, int n3, int r1, int r2, int nmf, int option, int order) {
  DefaultFpEnv fpenv;
  return orc::somf3d<double>(d, p1, p2, out, n1, n2, n3, r1, r2, nmf, option, order);
}

// Median of a given spray panel set u[ntr][np][n1], row `row`, window nmf
// (the selection step alone, for the bit-exact median check).
int orc_spray_median_f32(const float* u, float* out, int n1, int np, long ntr, int nmf,
                         int option) {
  DefaultFpEnv fpenv;
  if (n1 < 1 || np < 1 || nmf < 1 || (option != 1 && nmf < 5)) return orc::ORC_EINVAL;
  orc::SprayMedian<float> med;
  med.init(n1, np, nmf, option);
  for (long i = 0; i < ntr; i++) med.apply(u + i * np * n1, (np - 1) / 2, out + i * n1);
  return 0;
}

int orc_soint3d_f32(const float* din, const float* mask, const float* pp, const float* qq,
                    float* out, int n1, int n2, int n3, int nw, int nj1, int nj2, int niter,
                    int drift, int seed, int hasmask, float var) {
  DefaultFpEnv fpenv;
  return orc::soint3d<float>(din, mask, pp, qq, out, n1, n2, n3, nw, nj1, nj2, niter, drift, seed,
                             hasmask, var);
}
int orc_soint3d_f64(const double* din, const double* mask, const double* pp, const double* qq,
                    double* out, int n1, int n2, int n3, int nw, int nj1, int nj2, int niter,
                    int drift, int seed, int hasmask, double var) {
  DefaultFpEnv fpenv;
  return orc::soint3d<double>(din, mask, pp, qq, out, n1, n2, n3, nw, nj1, nj2, niter, drift,
                              seed, hasmask, var);
}

int orc_soint2d_prec_f32(const float* din, const float* mask, const float* pp, const float* qq,
                         float* out, int n1, int n2, int nw, int niter, int hasmask) {
  DefaultFpEnv fpenv;
  return orc::soint2d_prec<float>(din, mask, pp, qq, out, n1, n2, nw, niter, hasmask);
}
int orc_soint2d_prec_f64(const double* din, const double* mask, const double* pp,
                         const double* qq, double* out, int n1, int n2, int nw, int niter,
                         int hasmask) {
  DefaultFpEnv fpenv;
  return orc::soint2d_prec<double>(din, mask, pp, qq, out, n1, n2, nw, niter, hasmask);
}

int orc_bandpass_f32(const float* in, float* out, int n1, long ntr, float d1, float flo,
                     float fhi, int nplo, int nphi, int phase) {
  DefaultFpEnv fpenv;
  return orc::bandpass(in, out, n1, ntr, d1, flo, fhi, nplo, nphi, phase);
}

}  // extern "C"
