// FK dip filter: the work of one GPU thread in each pass, shared by the
// kernels of pwd_fk.cu and by the CPU test that runs this same code for
// every thread index (the header compiles as plain C++ without nvcc).
//
// Restates fkdip (pyseistr/fk.py:2-68), the cone-passed part of a section's
// FK spectrum back in time and space (the DAS chain subtracts it, demos/
// test_pyseistr_das.py:50):
//   1. FFT along time of every trace, zero-padded to nf = nextpow2(n1), in
//      the input's precision (numpy keeps float32 in complex64); rows
//      0 .. nf/2 kept (nrow = nf/2 + 1);
//   2. FFT along space of every kept row, zero-padded to nk = nextpow2(n2),
//      same precision;
//   3. the cone mask of the k = 0-centred plane (fftshift), whose float64
//      0/1 values promote the spectrum to complex128:
//      keep (i1, i2) (1-based, shifted column) when
//      i1 > (nrow / (w nk)) (i2 - nk/2) and i1 > (nrow / (w nk)) (nk/2 - i2);
//   4. inverse FFT along space (complex128, 1/nk);
//   5. the negative frequencies rebuilt as the conjugates of rows
//      nf/2 - 1 .. 1, inverse FFT along time (complex128, 1/nf), real part,
//      cut to n1 x n2.
// The FFTs are radix-2 Stockham passes (each pass reads one buffer and
// writes the other; log2 N passes leave the transform in natural order)
// with twiddles exp(-+2 pi i m / N) from a table computed once in double.
#pragma once

#ifdef __CUDACC__
#define PWD_FK_HD __host__ __device__ __forceinline__
#else
#define PWD_FK_HD inline
#endif

namespace pwd {
namespace fk {

template <class R>
struct Cx {
  R re, im;
};

template <class R>
PWD_FK_HD Cx<R> cmul(Cx<R> a, Cx<R> b) {
  Cx<R> c;
  c.re = a.re * b.re - a.im * b.im;
  c.im = a.re * b.im + a.im * b.re;
  return c;
}

PWD_FK_HD int pow2_at_least(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

// Step 1 input: element idx = b * nf + t of the [n2][nf] buffer.
template <class R, class T>
PWD_FK_HD void load_trace_sample(const T* d, Cx<R>* a, int n1, int nf, long idx) {
  const long b = idx / nf;
  const int t = (int)(idx - b * nf);
  Cx<R> v;
  v.re = t < n1 ? (R)d[b * n1 + t] : (R)0;
  v.im = (R)0;
  a[idx] = v;
}

// One radix-2 Stockham pass over a batch of transforms of length n stored
// one after another: butterfly idx = batch * (n/2) + j, sub-transform size
// ns (1, 2, 4, ... n/2).  tw[m] = exp(-2 pi i m / n), m < n/2; inverse
// passes use its conjugate.
template <class R>
PWD_FK_HD void stockham_pass(const Cx<R>* x, Cx<R>* y, int n, int ns, long idx,
                             const Cx<R>* tw, bool inverse) {
  const int h = n / 2;
  const long b = idx / h;
  const int j = (int)(idx - b * h);
  const Cx<R>* xs = x + b * n;
  Cx<R>* ys = y + b * n;
  const int k = j % ns;
  Cx<R> w = tw[k * (h / ns)];
  if (inverse) w.im = -w.im;
  const Cx<R> v0 = xs[j];
  const Cx<R> v1 = cmul(xs[j + h], w);
  const int o = (j / ns) * 2 * ns + k;
  Cx<R> s, t;
  s.re = v0.re + v1.re;
  s.im = v0.im + v1.im;
  t.re = v0.re - v1.re;
  t.im = v0.im - v1.im;
  ys[o] = s;
  ys[o + ns] = t;
}

// Step 2 input: element idx = f * nk + k of the [nrow][nk] buffer from the
// [n2][nf] time spectra.
template <class R>
PWD_FK_HD void rows_sample(const Cx<R>* a, Cx<R>* b, int n2, int nf, int nk, long idx) {
  const long f = idx / nk;
  const int k = (int)(idx - f * nk);
  Cx<R> v;
  v.re = (R)0;
  v.im = (R)0;
  if (k < n2) v = a[(long)k * nf + f];
  b[idx] = v;
}

// Step 3: the cone test of 0-based row f and shifted column c.
PWD_FK_HD bool cone_keeps(int f, int c, int nrow, int nk, double w) {
  const double s = (double)nrow / (w * (double)nk);
  const int half = nk / 2;
  const double i1 = (double)(f + 1);
  const int i2 = c + 1;
  return i1 > s * (double)(i2 - half) && i1 > s * (double)(half - i2);
}

// Step 3 on the unshifted spectrum: column k sits at shifted column
// (k + nk/2) mod nk (fftshift and ifftshift coincide for even nk; nk = 1
// has one column).
template <class R>
PWD_FK_HD void mask_sample(const Cx<R>* b, Cx<double>* c, int nrow, int nk, double w, long idx) {
  const long f = idx / nk;
  const int k = (int)(idx - f * nk);
  const int sc = (k + nk / 2) % nk;
  Cx<double> v;
  v.re = 0.;
  v.im = 0.;
  if (cone_keeps((int)f, sc, nrow, nk, w)) {
    v.re = (double)b[idx].re;
    v.im = (double)b[idx].im;
  }
  c[idx] = v;
}

// Step 5 input: element idx = k * nf + t of the [n2][nf] buffer (only the
// n2 output traces), rows scaled by 1/nk (the inverse space FFT's factor),
// negative frequencies conjugated.
PWD_FK_HD void full_sample(const Cx<double>* c, Cx<double>* dd, int nf, int nk, int nrow, long idx,
                           double inv_nk) {
  const long k = idx / nf;
  const int t = (int)(idx - k * nf);
  Cx<double> v;
  if (t < nrow) {
    v = c[(long)t * nk + k];
    v.re = v.re * inv_nk;
    v.im = v.im * inv_nk;
  } else {
    v = c[(long)(nf - t) * nk + k];
    v.re = v.re * inv_nk;
    v.im = -(v.im * inv_nk);
  }
  dd[idx] = v;
}

// Output sample idx = k * n1 + t: the real part of the inverse time FFT
// times 1/nf.
PWD_FK_HD void out_sample(const Cx<double>* dd, double* out, int n1, int nf, long idx,
                          double inv_nf) {
  const long k = idx / n1;
  const int t = (int)(idx - k * n1);
  out[idx] = dd[k * nf + t].re * inv_nf;
}

}  // namespace fk
}  // namespace pwd
