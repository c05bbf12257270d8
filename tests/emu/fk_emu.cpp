// Test harness: the FK dip filter's per-thread code
// (pyseistr_gb300/csrc/pwd_fk.cuh) run on the CPU for every element and
// butterfly of each pass, in the order of pwd_fk.cu's launches and with its
// twiddle tables, so that the CPU tests check the kernels' index arithmetic
// and FFT passes against the oracle.  Not part of the library.
#include <math.h>

#include <vector>

#include "../../pyseistr_gb300/csrc/pwd_fk.cuh"

namespace {

using pwd::fk::Cx;

void twiddles(int n, std::vector<double>& re, std::vector<double>& im) {
  re.clear();
  im.clear();
  for (int m = 0; m < n / 2; m++) {
    const double a = 2.0 * 3.14159265358979323846 * (double)m / (double)n;
    re.push_back(cos(a));
    im.push_back(-sin(a));
  }
}

template <class R>
Cx<R>* fft_batch(Cx<R>* x, Cx<R>* y, int len, long batch, const Cx<R>* tw, bool inverse) {
  const long nbf = batch * (len / 2);
  for (int ns = 1; ns < len; ns *= 2) {
    for (long i = 0; i < nbf; i++) pwd::fk::stockham_pass<R>(x, y, len, ns, i, tw, inverse);
    Cx<R>* t = x;
    x = y;
    y = t;
  }
  return x;
}

template <class R, class T>
int run(const T* d, double* out, int n1, int n2, double w) {
  if (n1 < 1 || n2 < 1 || w == 0.0) return 1;
  const int nf = pwd::fk::pow2_at_least(n1), nk = pwd::fk::pow2_at_least(n2);
  const int nrow = nf / 2 + 1;
  const long na = (long)n2 * nf, nb = (long)nrow * nk, no = (long)n1 * n2;
  std::vector<Cx<R>> a0(na), a1(na), b0(nb), b1(nb);
  std::vector<Cx<double>> c0(nb), c1(nb), d0(na), d1(na);
  std::vector<double> tre, tim, kre, kim;
  twiddles(nf, tre, tim);
  twiddles(nk, kre, kim);
  std::vector<Cx<R>> twt, twk;
  std::vector<Cx<double>> dwt, dwk;
  for (size_t m = 0; m < tre.size(); m++) {
    twt.push_back(Cx<R>{(R)tre[m], (R)tim[m]});
    dwt.push_back(Cx<double>{tre[m], tim[m]});
  }
  for (size_t m = 0; m < kre.size(); m++) {
    twk.push_back(Cx<R>{(R)kre[m], (R)kim[m]});
    dwk.push_back(Cx<double>{kre[m], kim[m]});
  }
  twt.push_back(Cx<R>{(R)1, (R)0});
  twk.push_back(Cx<R>{(R)1, (R)0});
  dwt.push_back(Cx<double>{1., 0.});
  dwk.push_back(Cx<double>{1., 0.});
  for (long i = 0; i < na; i++) pwd::fk::load_trace_sample<R, T>(d, a0.data(), n1, nf, i);
  Cx<R>* a = fft_batch<R>(a0.data(), a1.data(), nf, n2, twt.data(), false);
  for (long i = 0; i < nb; i++) pwd::fk::rows_sample<R>(a, b0.data(), n2, nf, nk, i);
  Cx<R>* b = fft_batch<R>(b0.data(), b1.data(), nk, nrow, twk.data(), false);
  for (long i = 0; i < nb; i++) pwd::fk::mask_sample<R>(b, c0.data(), nrow, nk, w, i);
  Cx<double>* c = fft_batch<double>(c0.data(), c1.data(), nk, nrow, dwk.data(), true);
  for (long i = 0; i < na; i++)
    pwd::fk::full_sample(c, d0.data(), nf, nk, nrow, i, 1.0 / (double)nk);
  Cx<double>* dd = fft_batch<double>(d0.data(), d1.data(), nf, n2, dwt.data(), true);
  for (long i = 0; i < no; i++) pwd::fk::out_sample(dd, out, n1, nf, i, 1.0 / (double)nf);
  return 0;
}

}  // namespace

extern "C" int emu_fkdip(const float* d, double* out, int n1, int n2, double w) {
  return run<float, float>(d, out, n1, n2, w);
}

extern "C" int emu_fkdip_f64(const double* d, double* out, int n1, int n2, double w) {
  return run<double, double>(d, out, n1, n2, w);
}
