// Plane-wave painting: the work of one GPU thread, shared by the kernel of
// pwd_paint.cu and by the CPU test that runs this same code for every thread
// (the header compiles as plain C++ without nvcc).
//
// Restates cpaint2d (pyseistr/src/paint_cfuns.c:1861-1940, called by
// pwpaintc and rgt, rgt.py:4-87): the seed trace is placed at trace i0 and
// carried trace by trace to both ends by the PWD prediction step
// (predict_step :1247-1274 with predict_init's eps = eps2 = eps^2):
// leftwards (i2 = i0-1 .. 0) along the slope of the trace reached, with the
// unreversed filter; rightwards (i2 = i0+1 .. n2-1) along the slope of the
// trace before it, with the reversed filter.  One prediction step is
//   regularization (:1223-1239), pwd_define (forw, :453-497 of the same
//   filter code), ps_banded_define (LDL' of the symmetric band, band 2 nw),
//   pwd_set (forward, the band's diag array as its scratch), the four end
//   terms eps2 t, and ps_banded_solve,
// every float and double operation of the reference in its order (no
// contraction), so the painted section is bit-identical.
//
// The chain is serial along the traces and each step is serial along the
// trace (the LDL' factorisation and the two substitutions), so a thread
// paints one direction of one section; the two directions of a section are
// independent once the seed is in place.  The thread's band arrays and
// factor live in its slice of the caller's workspace; its trace is the
// output trace it is painting (copied from the previous one, then predicted
// in place).
#pragma once

#ifdef __CUDACC__
#define PWD_PAINT_HD __host__ __device__ __forceinline__
#else
#define PWD_PAINT_HD inline
#endif

namespace pwd {
namespace paint {

constexpr int kMaxNw = 4;  // accuracy orders 1..4
constexpr int kMaxNa = 2 * kMaxNw + 1;

struct PaintParams {
  const float* dip;   // [n2][n1] slopes
  const float* seed;  // [n1] seed trace
  float* out;         // [n2][n1] painted section
  float* ws;          // 2 thread slices of slice_floats(n1, nw) floats
  int n1, n2, nw, i0;
  float eps;              // eps^2 of the caller's eps (predict_init's e)
  double b[kMaxNa];       // all-pass filter constants (apfilt_init)
};

// Floats of one thread's slice: diag, offd[2nw], taps a[2nw+1], LDL' d and
// o[2nw], each n1 long.
PWD_PAINT_HD long slice_floats(int n1, int nw) {
  return (long)(2 + 4 * nw + 2 * nw + 1) * n1;
}

PWD_PAINT_HD int imin(int a, int b) { return a < b ? a : b; }

// passfilter (paint_cfuns.c, the dip_cfuns.c:863-881 code): tap k is b[k]
// times the float factors (nf - j - p) or (p + j + 1), multiplied in double
// and rounded to float.
PWD_PAINT_HD void pass_taps(const double* b, int nf, float p, float* a) {
  for (int k = 0; k <= nf; k++) {
    double ak = b[k];
    for (int j = 0; j < nf; j++) {
      const float f = j < nf - k ? (float)(nf - j) - p : (p + (float)j) + 1.f;
      ak *= (double)f;
    }
    a[k] = (float)ak;
  }
}

// One prediction step of `trace` (n1 samples, in place) along the slope
// trace pp; forw selects the reversed filter.
PWD_PAINT_HD void predict_step(const PaintParams& q, float* s, bool forw, float* trace,
                               const float* pp) {
  const int n = q.n1, nw = q.nw, nb = 2 * nw, na = 2 * nw + 1;
  float* diag = s;
  float* offd = diag + n;       // offd[m][i] at offd[m * n + i]
  float* a = offd + nb * n;     // a[j][i] at a[j * n + i]
  float* d = a + na * n;
  float* o = d + n;             // o[m][k] at o[m * n + k]
  const float eps = q.eps, eps2 = q.eps;

  // regularization
  for (int i = 0; i < n; i++) {
    diag[i] = (float)(6. * eps);
    offd[i] = (float)(-4. * eps);
    offd[n + i] = eps;
    for (int ib = 2; ib < nb; ib++) offd[ib * n + i] = 0.f;
  }
  diag[0] = diag[n - 1] = eps2 + eps;
  diag[1] = diag[n - 2] = (float)(eps2 + 5. * eps);
  offd[0] = offd[n - 2] = (float)(-2. * eps);

  // pwd_define: taps per sample (reversed when forw), then the band
  float bb[kMaxNa];
  for (int i = 0; i < n; i++) {
    pass_taps(q.b, nb, pp[i], bb);
    for (int j = 0; j < na; j++) a[j * n + i] = forw ? bb[na - 1 - j] : bb[j];
  }
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < na; j++) {
      const int k = i + j - nw;
      if (k >= nw && k < n - nw) {
        const float aj = a[j * n + k];
        diag[i] += aj * aj;
      }
    }
    for (int m = 0; m < nb; m++)
      for (int j = m + 1; j < na; j++) {
        const int k = i + j - nw;
        if (k >= nw && k < n - nw) {
          const float aj = a[j * n + k];
          const float am = a[(j - m - 1) * n + k];
          offd[m * n + i] += am * aj;
        }
      }
  }

  // ps_banded_define: LDL' of the band
  for (int k = 0; k < n; k++) {
    float t = diag[k];
    int m1 = imin(k, nb);
    for (int m = 0; m < m1; m++) {
      const float om = o[m * n + k - m - 1];
      t -= om * om * d[k - m - 1];
    }
    d[k] = t;
    const int nn1 = imin(n - k - 1, nb);
    for (int c = 0; c < nn1; c++) {
      t = offd[c * n + k];
      m1 = imin(k, nb - c - 1);
      for (int m = 0; m < m1; m++)
        t -= o[m * n + k - m - 1] * o[(c + m + 1) * n + k - m - 1] * d[k - m - 1];
      o[c * n + k] = t / d[k];
    }
  }

  // the four end values, then pwd_set (forward) with diag as its scratch
  const float t0 = trace[0], t1 = trace[1], t2 = trace[n - 2], t3 = trace[n - 1];
  float* tmp = diag;
  for (int i = 0; i < n; i++) tmp[i] = 0.f;
  for (int i = nw; i < n - nw; i++)
    for (int j = 0; j < na; j++) {
      const int k = i + j - nw;
      tmp[i] += a[j * n + i] * trace[k];
    }
  for (int i = 0; i < n; i++) {
    trace[i] = 0.f;
    for (int j = 0; j < na; j++) {
      const int k = i + j - nw;
      if (k >= nw && k < n - nw) trace[i] += a[j * n + k] * tmp[k];
    }
  }
  trace[0] += eps2 * t0;
  trace[1] += eps2 * t1;
  trace[n - 2] += eps2 * t2;
  trace[n - 1] += eps2 * t3;

  // ps_banded_solve
  for (int k = 1; k < n; k++) {
    float t = trace[k];
    const int m1 = imin(k, nb);
    for (int m = 0; m < m1; m++) t -= o[m * n + k - m - 1] * trace[k - m - 1];
    trace[k] = t;
  }
  for (int k = n - 1; k >= 0; k--) {
    float t = trace[k] / d[k];
    const int m1 = imin(n - k - 1, nb);
    for (int m = 0; m < m1; m++) t -= o[m * n + k] * trace[k + m + 1];
    trace[k] = t;
  }
}

// Thread `side` of the section: 0 places the seed and paints leftwards, 1
// paints rightwards (from the seed array, so that it does not wait on 0).
PWD_PAINT_HD void paint_side(const PaintParams& q, int side) {
  const int n = q.n1;
  float* s = q.ws + (long)side * slice_floats(n, q.nw);
  if (side == 0) {
    float* tr = q.out + (long)q.i0 * n;
    for (int i = 0; i < n; i++) tr[i] = q.seed[i];
    for (int i2 = q.i0 - 1; i2 >= 0; i2--) {
      float* t = q.out + (long)i2 * n;
      const float* prev = t + n;
      for (int i = 0; i < n; i++) t[i] = prev[i];
      predict_step(q, s, false, t, q.dip + (long)i2 * n);
    }
  } else {
    for (int i2 = q.i0 + 1; i2 < q.n2; i2++) {
      float* t = q.out + (long)i2 * n;
      const float* prev = i2 == q.i0 + 1 ? q.seed : t - n;
      for (int i = 0; i < n; i++) t[i] = prev[i];
      predict_step(q, s, true, t, q.dip + (long)(i2 - 1) * n);
    }
  }
}

// Stacked sections of one size: thread g paints side g % 2 of section g / 2
// (slopes and output at section * n1 n2, seed at section * n1, band arrays
// in slices 2 section and 2 section + 1 of the workspace).
PWD_PAINT_HD void paint_item(const PaintParams& q, long g) {
  const long sec = g / 2, n12 = (long)q.n1 * q.n2;
  PaintParams p = q;
  p.dip = q.dip + sec * n12;
  p.seed = q.seed + sec * q.n1;
  p.out = q.out + sec * n12;
  p.ws = q.ws + sec * 2 * slice_floats(q.n1, q.nw);
  paint_side(p, (int)(g - 2 * sec));
}

// apfilt_init (paint_cfuns.c, the dip_cfuns.c:835-855 code), in double.
inline void filter_constants(int nw, double* b) {
  const int nf = 2 * nw;
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

}  // namespace paint
}  // namespace pwd
