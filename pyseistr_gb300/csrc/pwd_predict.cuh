// One plane-wave-destruction trace prediction, streamed along the trace by
// one thread.
//
// Restates predict_step(adj=false) (pyseistr/src/sof_cfuns.c:622-649),
// predict1_step and predict2_step (sof3d_cfuns.c:596-661) and the adjoint
// predict_step(adj=true): regularization (:603-620), pwd_define (:453-497),
// sf_banded_define (:161-186), pwd_set (:499-555) and sf_banded_solve
// (:287-307), with the same float operations in the same order.
//
// The ascending pass keeps sliding windows (registers) of the filter
// columns, the pwd_set intermediate and the last `band` LDL' columns, and
// fuses the band accumulation, the factorisation, the filter application
// and the forward substitution; the descending pass does the back
// substitution.  The factor (o, d) and the forward-substituted trace (y)
// go to a per-thread, thread-interleaved scratch (element k at k*ss).
#pragma once

#include "pwd_common.cuh"

namespace pwd {

struct PredictScratch {
  float* o;  // [NB][n1] interleaved: o[m][k] at (m*n1 + k)*ss
  float* d;  // [n1]
  float* y;  // [n1]
  long ss;   // interleave stride (number of threads sharing the scratch)
};

template <int NW>
struct FilterWin {
  // a[c][j]: filter tap j of column (i - NW + c), c = 0..2NW
  float a[2 * NW + 1][2 * NW + 1];
};

template <int NW>
__device__ __forceinline__ void filter_column(const ApCoef& c, float p, bool reversed, float* col) {
  float b[2 * NW + 1];
  passfilter<NW>(c, p, b);
#pragma unroll
  for (int j = 0; j <= 2 * NW; j++) col[j] = reversed ? b[2 * NW - j] : b[j];
}

template <int NW>
__device__ __forceinline__ void shift_win(FilterWin<NW>& w) {
#pragma unroll
  for (int c = 0; c < 2 * NW; c++)
#pragma unroll
    for (int j = 0; j <= 2 * NW; j++) w.a[c][j] = w.a[c + 1][j];
}

// Band entries of row i from the filter window (pwd_define :475-495): adds
// to diag and offd[0..NB) in the reference's j order.
template <int NW>
__device__ __forceinline__ void band_add(const FilterWin<NW>& w, int i, int n1, float& diag,
                                         float* offd) {
  constexpr int NA = 2 * NW + 1, NB = 2 * NW;
#pragma unroll
  for (int j = 0; j < NA; j++) {
    int k = i + j - NW;
    if (k >= NW && k < n1 - NW) {
      float aj = w.a[j][j];
      diag = __fadd_rn(diag, __fmul_rn(aj, aj));
    }
  }
#pragma unroll
  for (int m = 0; m < NB; m++) {
#pragma unroll
    for (int j = m + 1; j < NA; j++) {
      int k = i + j - NW;
      if (k >= NW && k < n1 - NW) {
        float aj = w.a[j][j];
        float am = w.a[j][j - m - 1];
        offd[m] = __fadd_rn(offd[m], __fmul_rn(am, aj));
      }
    }
  }
}

// regularization() (sof_cfuns.c:603-620) constants, computed once per
// prediction: the reference evaluates 6.*eps, eps2+5.*eps, -4.*eps and
// -2.*eps in double and stores them as float.
struct RegConst {
  float d_mid, d_end, d_next, o_mid, o_end, o1;
};
__device__ __forceinline__ RegConst reg_const(float eps, float eps2) {
  RegConst r;
  r.d_mid = __double2float_rn(6. * (double)eps);
  r.d_end = __fadd_rn(eps2, eps);
  r.d_next = __double2float_rn((double)eps2 + 5. * (double)eps);
  r.o_mid = __double2float_rn(-4. * (double)eps);
  r.o_end = __double2float_rn(-2. * (double)eps);
  r.o1 = eps;
  return r;
}

// regularization() values of row i.
template <int NB>
__device__ __forceinline__ void reg_row(int i, int n1, const RegConst& rc, float& diag,
                                        float* offd) {
  diag = rc.d_mid;
  if (i == 0 || i == n1 - 1) diag = rc.d_end;
  if (i == 1 || i == n1 - 2) diag = rc.d_next;
  offd[0] = (i == 0 || i == n1 - 2) ? rc.o_end : rc.o_mid;
  offd[1] = rc.o1;
#pragma unroll
  for (int b = 2; b < NB; b++) offd[b] = 0.f;
}

// sf_banded_define step at row k with the window of previous columns:
// O[c][m] = o[m][k-1-c], D[c] = d[k-1-c].  Returns d[k] and o[0..NB)[k].
template <int NB>
__device__ __forceinline__ void ldl_row(int k, int n1, float diag, const float* offd,
                                        const float (&O)[NB][NB], const float (&D)[NB],
                                        float& dk, float* ok) {
  float t = diag;
#pragma unroll
  for (int m = 0; m < NB; m++)
    if (m < k) t = __fsub_rn(t, __fmul_rn(__fmul_rn(O[m][m], O[m][m]), D[m]));
  dk = t;
#pragma unroll
  for (int q = 0; q < NB; q++) {
    if (q < n1 - k - 1) {
      float s = offd[q];
#pragma unroll
      for (int m = 0; m < NB - q - 1; m++)
        if (m < k) s = __fsub_rn(s, __fmul_rn(__fmul_rn(O[m][m], O[m][q + m + 1]), D[m]));
      ok[q] = __fdiv_rn(s, dk);
    } else {
      ok[q] = 0.f;
    }
  }
}

// Forward prediction into `out` (predict_step adj=false, predict1_step,
// predict2_step).  in1/in2 input traces, pp1/pp2 slope traces, contiguous.
// forw1/forw2 select the reversed filter (pwd_define adj flag).
template <int NW, bool TWO>
__device__ void predict_fwd(int n1, float eps, float eps2, const ApCoef& c,
                            const float* __restrict__ in1, const float* __restrict__ pp1,
                            bool forw1, const float* __restrict__ in2,
                            const float* __restrict__ pp2, bool forw2, float* __restrict__ out,
                            const PredictScratch& sc) {
  constexpr int NA = 2 * NW + 1, NB = 2 * NW;
  const RegConst rc = reg_const(eps, eps2);
  FilterWin<NW> w1, w2;
  float x1[NA], x2[NA];  // input windows in[i .. i+2NW]
  float t1[NA], t2[NA];  // pwd_set intermediates tmp[i-NW .. i+NW]
  float O[NB][NB], D[NB];  // previous LDL' columns
  float Y[NB];             // previous forward-substituted values y[k-1-c]

#pragma unroll
  for (int cc = 0; cc < NA; cc++)
#pragma unroll
    for (int j = 0; j < NA; j++) {
      w1.a[cc][j] = 0.f;
      if (TWO) w2.a[cc][j] = 0.f;
    }
#pragma unroll
  for (int cc = 0; cc < NA; cc++) {
    t1[cc] = 0.f;
    t2[cc] = 0.f;
  }
#pragma unroll
  for (int m = 0; m < NB; m++) {
    D[m] = 0.f;
    Y[m] = 0.f;
#pragma unroll
    for (int q = 0; q < NB; q++) O[m][q] = 0.f;
  }
  // prefill: filter columns 0..NW-1 go to window slots NW+1..2NW (for i=0 the
  // window holds columns -NW..NW); inputs in[0..2NW-1] to x slots 1..2NW.
#pragma unroll
  for (int cc = 0; cc < NW; cc++) {
    if (cc < n1) {
      filter_column<NW>(c, pp1[cc], forw1, w1.a[NW + 1 + cc]);
      if (TWO) filter_column<NW>(c, pp2[cc], forw2, w2.a[NW + 1 + cc]);
    }
  }
#pragma unroll
  for (int q = 0; q < NB; q++) {
    x1[q + 1] = q < n1 ? in1[q] : 0.f;
    if (TWO) x2[q + 1] = q < n1 ? in2[q] : 0.f;
  }
  float b0, b1, b2, b3;  // boundary values t0..t3
  if (TWO) {
    b0 = __fmul_rn(0.5f, __fadd_rn(in1[0], in2[0]));
    b1 = __fmul_rn(0.5f, __fadd_rn(in1[1], in2[1]));
    b2 = __fmul_rn(0.5f, __fadd_rn(in1[n1 - 2], in2[n1 - 2]));
    b3 = __fmul_rn(0.5f, __fadd_rn(in1[n1 - 1], in2[n1 - 1]));
  } else {
    b0 = in1[0];
    b1 = in1[1];
    b2 = in1[n1 - 2];
    b3 = in1[n1 - 1];
  }

  for (int i = 0; i < n1; i++) {
    // advance: column i+NW enters the windows
    const int cn = i + NW;
    shift_win<NW>(w1);
    if (TWO) shift_win<NW>(w2);
#pragma unroll
    for (int q = 0; q < NA - 1; q++) {
      x1[q] = x1[q + 1];
      t1[q] = t1[q + 1];
      if (TWO) {
        x2[q] = x2[q + 1];
        t2[q] = t2[q + 1];
      }
    }
    const int ln = i + 2 * NW;  // newest input sample
    x1[NA - 1] = ln < n1 ? in1[ln] : 0.f;
    if (TWO) x2[NA - 1] = ln < n1 ? in2[ln] : 0.f;
    if (cn < n1) {
      filter_column<NW>(c, pp1[cn], forw1, w1.a[2 * NW]);
      if (TWO) filter_column<NW>(c, pp2[cn], forw2, w2.a[2 * NW]);
    } else {
#pragma unroll
      for (int j = 0; j < NA; j++) {
        w1.a[2 * NW][j] = 0.f;
        if (TWO) w2.a[2 * NW][j] = 0.f;
      }
    }
    // pwd_set forward, first loop: tmp[cn] = sum_j a[j][cn] * in[cn+j-NW]
    float s1 = 0.f, s2 = 0.f;
    if (cn >= NW && cn < n1 - NW) {
#pragma unroll
      for (int j = 0; j < NA; j++) {
        s1 = __fadd_rn(s1, __fmul_rn(w1.a[2 * NW][j], x1[j]));
        if (TWO) s2 = __fadd_rn(s2, __fmul_rn(w2.a[2 * NW][j], x2[j]));
      }
    }
    t1[NA - 1] = s1;
    if (TWO) t2[NA - 1] = s2;

    // band row i: regularization + pwd_define of each filter
    float diag, offd[NB];
    reg_row<NB>(i, n1, rc, diag, offd);
    band_add<NW>(w1, i, n1, diag, offd);
    if (TWO) band_add<NW>(w2, i, n1, diag, offd);

    // pwd_set forward, second loop: out[i] = sum_j a[j][k] tmp[k], k=i+j-NW
    float o1 = 0.f, o2 = 0.f;
#pragma unroll
    for (int j = 0; j < NA; j++) {
      int k = i + j - NW;
      if (k >= NW && k < n1 - NW) {
        o1 = __fadd_rn(o1, __fmul_rn(w1.a[j][j], t1[j]));
        if (TWO) o2 = __fadd_rn(o2, __fmul_rn(w2.a[j][j], t2[j]));
      }
    }
    float b = TWO ? __fadd_rn(o1, o2) : o1;
    if (i == 0) b = __fadd_rn(b, __fmul_rn(eps2, b0));
    if (i == 1) b = __fadd_rn(b, __fmul_rn(eps2, b1));
    if (i == n1 - 2) b = __fadd_rn(b, __fmul_rn(eps2, b2));
    if (i == n1 - 1) b = __fadd_rn(b, __fmul_rn(eps2, b3));

    // LDL' row and forward substitution
    float dk, ok[NB];
    ldl_row<NB>(i, n1, diag, offd, O, D, dk, ok);
    float y = b;
#pragma unroll
    for (int m = 0; m < NB; m++)
      if (m < i) y = __fsub_rn(y, __fmul_rn(O[m][m], Y[m]));
    // store the factor column and y for the descending pass
#pragma unroll
    for (int m = 0; m < NB; m++) sc.o[((long)m * n1 + i) * sc.ss] = ok[m];
    sc.d[(long)i * sc.ss] = dk;
    sc.y[(long)i * sc.ss] = y;
    // shift the LDL' windows: column i becomes c=0
#pragma unroll
    for (int m = NB - 1; m > 0; m--) {
      D[m] = D[m - 1];
      Y[m] = Y[m - 1];
#pragma unroll
      for (int q = 0; q < NB; q++) O[m][q] = O[m - 1][q];
    }
    D[0] = dk;
    Y[0] = y;
#pragma unroll
    for (int q = 0; q < NB; q++) O[0][q] = ok[q];
  }

  // back substitution: x[k] = y[k]/d[k] - sum_m o[m][k] x[k+m+1]
  float X[NB];
#pragma unroll
  for (int m = 0; m < NB; m++) X[m] = 0.f;
  for (int k = n1 - 1; k >= 0; k--) {
    const float dk = sc.d[(long)k * sc.ss];
    float t = __fdiv_rn(sc.y[(long)k * sc.ss], dk);
#pragma unroll
    for (int m = 0; m < NB; m++)
      if (m < n1 - k - 1) t = __fsub_rn(t, __fmul_rn(sc.o[((long)m * n1 + k) * sc.ss], X[m]));
#pragma unroll
    for (int m = NB - 1; m > 0; m--) X[m] = X[m - 1];
    X[0] = t;
    out[k] = t;
  }
}

// ---------------------------------------------------------------------------
// Factor once, apply many times.  The band matrix of a prediction into a
// trace (regularization + pwd_define of one filter) depends only on the
// slopes used and the filter orientation, not on the trace predicted, so
// every chain step of the spray that uses the slopes of trace k with
// orientation forw shares one LDL' factor.  PredictFactor holds, for one
// slope trace, its passfilter taps and the factors of both orientations,
// element (m, i) at (m*n1 + i)*ss (ss = traces sharing the store).
// ---------------------------------------------------------------------------
struct PredictFactor {
  float* taps;  // [NA][n1]  passfilter taps of each sample, unreversed
  float* f0;    // [NB+1][n1] forw = false: o[0..NB) then d
  float* f1;    // [NB+1][n1] forw = true
  long ss;
};

// Taps and both factors of one slope trace pp (the band and LDL' steps of
// predict_fwd with one filter, for the two orientations side by side, the
// taps of each column evaluated once for both).
template <int NW>
__device__ void predict_factor_pair(int n1, float eps, float eps2, const ApCoef& c,
                               const float* __restrict__ pp, const PredictFactor& F) {
  constexpr int NA = 2 * NW + 1, NB = 2 * NW;
  const RegConst rc = reg_const(eps, eps2);
  FilterWin<NW> wa, wb;  // unreversed / reversed columns
  float Oa[NB][NB], Da[NB], Ob[NB][NB], Db[NB];
#pragma unroll
  for (int cc = 0; cc < NA; cc++)
#pragma unroll
    for (int j = 0; j < NA; j++) {
      wa.a[cc][j] = 0.f;
      wb.a[cc][j] = 0.f;
    }
#pragma unroll
  for (int m = 0; m < NB; m++) {
    Da[m] = 0.f;
    Db[m] = 0.f;
#pragma unroll
    for (int q = 0; q < NB; q++) {
      Oa[m][q] = 0.f;
      Ob[m][q] = 0.f;
    }
  }
  auto column = [&](int cn, float* ca, float* cb) {
    float t[NA];
    passfilter<NW>(c, pp[cn], t);
#pragma unroll
    for (int j = 0; j < NA; j++) {
      F.taps[((long)j * n1 + cn) * F.ss] = t[j];
      ca[j] = t[j];
      cb[j] = t[NA - 1 - j];
    }
  };
#pragma unroll
  for (int cc = 0; cc < NW; cc++)
    if (cc < n1) column(cc, wa.a[NW + 1 + cc], wb.a[NW + 1 + cc]);
  for (int i = 0; i < n1; i++) {
    const int cn = i + NW;
    shift_win<NW>(wa);
    shift_win<NW>(wb);
    if (cn < n1) {
      column(cn, wa.a[2 * NW], wb.a[2 * NW]);
    } else {
#pragma unroll
      for (int j = 0; j < NA; j++) {
        wa.a[2 * NW][j] = 0.f;
        wb.a[2 * NW][j] = 0.f;
      }
    }
#pragma unroll
    for (int side = 0; side < 2; side++) {
      float diag, offd[NB];
      reg_row<NB>(i, n1, rc, diag, offd);
      band_add<NW>(side ? wb : wa, i, n1, diag, offd);
      float dk, ok[NB];
      ldl_row<NB>(i, n1, diag, offd, side ? Ob : Oa, side ? Db : Da, dk, ok);
      float* f = side ? F.f1 : F.f0;
#pragma unroll
      for (int m = 0; m < NB; m++) f[((long)m * n1 + i) * F.ss] = ok[m];
      f[((long)NB * n1 + i) * F.ss] = dk;
      float(&O)[NB][NB] = side ? Ob : Oa;
      float(&D)[NB] = side ? Db : Da;
#pragma unroll
      for (int m = NB - 1; m > 0; m--) {
        D[m] = D[m - 1];
#pragma unroll
        for (int q = 0; q < NB; q++) O[m][q] = O[m - 1][q];
      }
      D[0] = dk;
#pragma unroll
      for (int q = 0; q < NB; q++) O[0][q] = ok[q];
    }
  }
}

// One factor of slope trace pp (the band and LDL' steps of predict_fwd with
// one filter): side 0 the unreversed filter (forw = false, into F.f0, also
// storing the taps), side 1 the reversed one (F.f1; the taps too when
// with_taps).  The two sides are independent and run on two threads.
template <int NW>
__device__ void predict_factor(int n1, float eps, float eps2, const ApCoef& c,
                               const float* __restrict__ pp, const PredictFactor& F, int side,
                               bool with_taps = false) {
  constexpr int NA = 2 * NW + 1, NB = 2 * NW;
  const RegConst rc = reg_const(eps, eps2);
  FilterWin<NW> w;
  float O[NB][NB], D[NB];
#pragma unroll
  for (int cc = 0; cc < NA; cc++)
#pragma unroll
    for (int j = 0; j < NA; j++) w.a[cc][j] = 0.f;
#pragma unroll
  for (int m = 0; m < NB; m++) {
    D[m] = 0.f;
#pragma unroll
    for (int q = 0; q < NB; q++) O[m][q] = 0.f;
  }
  float* f = side ? F.f1 : F.f0;
  auto column = [&](int cn, float* col) {
    float t[NA];
    passfilter<NW>(c, pp[cn], t);
#pragma unroll
    for (int j = 0; j < NA; j++) {
      if (side == 0 || with_taps) F.taps[((long)j * n1 + cn) * F.ss] = t[j];
      col[j] = side ? t[NA - 1 - j] : t[j];
    }
  };
#pragma unroll
  for (int cc = 0; cc < NW; cc++)
    if (cc < n1) column(cc, w.a[NW + 1 + cc]);
  for (int i = 0; i < n1; i++) {
    const int cn = i + NW;
    shift_win<NW>(w);
    if (cn < n1) {
      column(cn, w.a[2 * NW]);
    } else {
#pragma unroll
      for (int j = 0; j < NA; j++) w.a[2 * NW][j] = 0.f;
    }
    float diag, offd[NB];
    reg_row<NB>(i, n1, rc, diag, offd);
    band_add<NW>(w, i, n1, diag, offd);
    float dk, ok[NB];
    ldl_row<NB>(i, n1, diag, offd, O, D, dk, ok);
#pragma unroll
    for (int m = 0; m < NB; m++) f[((long)m * n1 + i) * F.ss] = ok[m];
    f[((long)NB * n1 + i) * F.ss] = dk;
#pragma unroll
    for (int m = NB - 1; m > 0; m--) {
      D[m] = D[m - 1];
#pragma unroll
      for (int q = 0; q < NB; q++) O[m][q] = O[m - 1][q];
    }
    D[0] = dk;
#pragma unroll
    for (int q = 0; q < NB; q++) O[0][q] = ok[q];
  }
}

// Forward prediction (predict_step adj=false) of in1 (and, with RHS2, of
// in1b through the same factor) with a precomputed factor: pwd_set with the
// stored taps (reversed when forw), the eps2 boundary terms, forward and
// back substitution.  The operations on the trace are those of predict_fwd.
// taps/fac point at the slope trace's column 0 with stride fss; ys is the
// chain's scratch (element k at k*yss) for y (and yb).  The inputs are read
// with strides ins/insb; the back substitution leaves the predicted trace
// in ys (ysb) as well as in out (outb), so that the next step of a chain
// reads its input from the chain-interleaved scratch (coalesced across a
// warp) rather than from the sprayed panel.  Every operand of a
// sample (taps, factor elements, input, y) is staged kApplyStages - 1
// samples ahead by cp.async into the thread's ring in shared memory: ring
// element e of slot q at ring[(q*apply_elems(NW) + e)*rs] (rs = threads of the
// block, so consecutive threads hit consecutive banks).  IX is the type of
// the element offsets: int where every offset of the section's factor store
// fits in 32 bits (fewer integer instructions a sample), long otherwise.
#ifndef PWD_APPLY_STAGES
#define PWD_APPLY_STAGES 4
#endif
constexpr int kApplyStages = PWD_APPLY_STAGES;
__host__ __device__ constexpr int apply_elems(int nw) { return 4 * nw + 3; }  // NA + NB + 2

template <int NW, bool RHS2, typename IX = long>
__device__ void predict_apply(int n1, float eps2, const float* __restrict__ taps,
                              const float* __restrict__ fac, IX fss, bool forw,
                              const float* in1, IX ins, float* __restrict__ out, float* ys,
                              float* ysb, IX yss, float* ring, int rs,
                              const float* in1b = nullptr, IX insb = 1,
                              float* __restrict__ outb = nullptr) {
  constexpr int NA = 2 * NW + 1, NB = 2 * NW, P = kApplyStages, NE = apply_elems(NW);
  // the input trace (the previous step's output) and, below, the y scratch
  // were written by this thread's ordinary stores; order them before the
  // asynchronous copies that read them back
  __threadfence_block();
  FilterWin<NW> w1;
  float x1[NA], xb[NA], t1[NA], tb[NA], Y[NB], YB[NB];
#pragma unroll
  for (int cc = 0; cc < NA; cc++) {
    t1[cc] = 0.f;
    tb[cc] = 0.f;
#pragma unroll
    for (int j = 0; j < NA; j++) w1.a[cc][j] = 0.f;
  }
#pragma unroll
  for (int m = 0; m < NB; m++) {
    Y[m] = 0.f;
    YB[m] = 0.f;
  }
  auto R = [&](int q, int e) -> float* { return ring + (q * NE + e) * rs; };
  auto set_col = [&](const float* v, float* col) {
#pragma unroll
    for (int j = 0; j < NA; j++) col[j] = forw ? v[NA - 1 - j] : v[j];
  };
#pragma unroll
  for (int cc = 0; cc < NW; cc++)
    if (cc < n1) {
      float v[NA];
#pragma unroll
      for (int j = 0; j < NA; j++) v[j] = taps[((IX)j * n1 + cc) * fss];
      set_col(v, w1.a[NW + 1 + cc]);
    }
#pragma unroll
  for (int q = 0; q < NB; q++) {
    x1[q + 1] = q < n1 ? in1[q * ins] : 0.f;
    if (RHS2) xb[q + 1] = q < n1 ? in1b[q * insb] : 0.f;
  }
  const float b0 = in1[0], b1 = in1[ins], b2 = in1[(n1 - 2) * ins], b3 = in1[(n1 - 1) * ins];
  float c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f;
  if (RHS2) {
    c0 = in1b[0];
    c1 = in1b[insb];
    c2 = in1b[(n1 - 2) * insb];
    c3 = in1b[(n1 - 1) * insb];
  }
  // forward pass operands of sample i: taps of column i+NW (0..NA), factor
  // o[m][i-1-m] (NA..NA+NB), inputs in[i+2NW] (NA+NB, +1)
  auto stage_f = [&](int i) {
    if (i < n1) {
      const int q = i % P, cn = i + NW, ln = i + 2 * NW;
      if (cn < n1)
#pragma unroll
        for (int j = 0; j < NA; j++) cp_async4(R(q, j), taps + ((IX)j * n1 + cn) * fss);
#pragma unroll
      for (int m = 0; m < NB; m++)
        if (m < i) cp_async4(R(q, NA + m), fac + ((IX)m * n1 + (i - 1 - m)) * fss);
      if (ln < n1) {
        cp_async4(R(q, NA + NB), in1 + ln * ins);
        if (RHS2) cp_async4(R(q, NA + NB + 1), in1b + ln * insb);
      }
    }
    cp_async_commit();
  };
#pragma unroll
  for (int k = 0; k < P - 1; k++) stage_f(k);
  for (int i = 0; i < n1; i++) {
    stage_f(i + P - 1);
    cp_async_wait<P - 1>();
    const int q = i % P;
    const int cn = i + NW;
    shift_win<NW>(w1);
#pragma unroll
    for (int qq = 0; qq < NA - 1; qq++) {
      x1[qq] = x1[qq + 1];
      t1[qq] = t1[qq + 1];
      if (RHS2) {
        xb[qq] = xb[qq + 1];
        tb[qq] = tb[qq + 1];
      }
    }
    const int ln = i + 2 * NW;
    x1[NA - 1] = ln < n1 ? *R(q, NA + NB) : 0.f;
    if (RHS2) xb[NA - 1] = ln < n1 ? *R(q, NA + NB + 1) : 0.f;
    if (cn < n1) {
      float v[NA];
#pragma unroll
      for (int j = 0; j < NA; j++) v[j] = *R(q, j);
      set_col(v, w1.a[2 * NW]);
    } else {
#pragma unroll
      for (int j = 0; j < NA; j++) w1.a[2 * NW][j] = 0.f;
    }
    float s1 = 0.f, sb = 0.f;
    if (cn >= NW && cn < n1 - NW) {
#pragma unroll
      for (int j = 0; j < NA; j++) {
        s1 = __fadd_rn(s1, __fmul_rn(w1.a[2 * NW][j], x1[j]));
        if (RHS2) sb = __fadd_rn(sb, __fmul_rn(w1.a[2 * NW][j], xb[j]));
      }
    }
    t1[NA - 1] = s1;
    if (RHS2) tb[NA - 1] = sb;
    float o1 = 0.f, ob = 0.f;
#pragma unroll
    for (int j = 0; j < NA; j++) {
      int k = i + j - NW;
      if (k >= NW && k < n1 - NW) {
        o1 = __fadd_rn(o1, __fmul_rn(w1.a[j][j], t1[j]));
        if (RHS2) ob = __fadd_rn(ob, __fmul_rn(w1.a[j][j], tb[j]));
      }
    }
    float b = o1;
    if (i == 0) b = __fadd_rn(b, __fmul_rn(eps2, b0));
    if (i == 1) b = __fadd_rn(b, __fmul_rn(eps2, b1));
    if (i == n1 - 2) b = __fadd_rn(b, __fmul_rn(eps2, b2));
    if (i == n1 - 1) b = __fadd_rn(b, __fmul_rn(eps2, b3));
    if (RHS2) {
      if (i == 0) ob = __fadd_rn(ob, __fmul_rn(eps2, c0));
      if (i == 1) ob = __fadd_rn(ob, __fmul_rn(eps2, c1));
      if (i == n1 - 2) ob = __fadd_rn(ob, __fmul_rn(eps2, c2));
      if (i == n1 - 1) ob = __fadd_rn(ob, __fmul_rn(eps2, c3));
    }
    // forward substitution with o[m][i-1-m] of the stored factor
    float y = b, y2 = ob;
#pragma unroll
    for (int m = 0; m < NB; m++)
      if (m < i) {
        const float om = *R(q, NA + m);
        y = __fsub_rn(y, __fmul_rn(om, Y[m]));
        if (RHS2) y2 = __fsub_rn(y2, __fmul_rn(om, YB[m]));
      }
    ys[(IX)i * yss] = y;
    if (RHS2) ysb[(IX)i * yss] = y2;
#pragma unroll
    for (int m = NB - 1; m > 0; m--) {
      Y[m] = Y[m - 1];
      if (RHS2) YB[m] = YB[m - 1];
    }
    Y[0] = y;
    if (RHS2) YB[0] = y2;
  }
  cp_async_wait<0>();
  __threadfence_block();
  // back substitution: x[k] = y[k]/d[k] - sum_m o[m][k] x[k+m+1]; operands
  // of row k: o[m][k] (0..NB), d[k] (NB), y[k] (NB+1), yb[k] (NB+2).  The
  // scratch y written above by this thread is complete (program order).
  auto stage_b = [&](int step) {
    if (step < n1) {
      const int k = n1 - 1 - step, q = step % P;
#pragma unroll
      for (int m = 0; m < NB; m++)
        if (m < n1 - k - 1) cp_async4(R(q, m), fac + ((IX)m * n1 + k) * fss);
      cp_async4(R(q, NB), fac + ((IX)NB * n1 + k) * fss);
      cp_async4(R(q, NB + 1), ys + (IX)k * yss);
      if (RHS2) cp_async4(R(q, NB + 2), ysb + (IX)k * yss);
    }
    cp_async_commit();
  };
  float X[NB], XB[NB];
#pragma unroll
  for (int m = 0; m < NB; m++) {
    X[m] = 0.f;
    XB[m] = 0.f;
  }
#pragma unroll
  for (int k = 0; k < P - 1; k++) stage_b(k);
  for (int step = 0; step < n1; step++) {
    stage_b(step + P - 1);
    cp_async_wait<P - 1>();
    const int k = n1 - 1 - step, q = step % P;
    const float dk = *R(q, NB);
    float t = __fdiv_rn(*R(q, NB + 1), dk);
    float tb2 = RHS2 ? __fdiv_rn(*R(q, NB + 2), dk) : 0.f;
#pragma unroll
    for (int m = 0; m < NB; m++)
      if (m < n1 - k - 1) {
        const float om = *R(q, m);
        t = __fsub_rn(t, __fmul_rn(om, X[m]));
        if (RHS2) tb2 = __fsub_rn(tb2, __fmul_rn(om, XB[m]));
      }
#pragma unroll
    for (int m = NB - 1; m > 0; m--) {
      X[m] = X[m - 1];
      if (RHS2) XB[m] = XB[m - 1];
    }
    X[0] = t;
    out[k] = t;
    ys[(IX)k * yss] = t;  // y[k] is consumed: the slot carries the output
    if (RHS2) {
      XB[0] = tb2;
      outb[k] = tb2;
      ysb[(IX)k * yss] = tb2;
    }
  }
  cp_async_wait<0>();
}

// Adjoint prediction in place with a stored factor (predict_step adj=true,
// sof_cfuns.c:622-649, with the factor k_spray2_factor stored): the banded
// solve with the stored LDL' factor, the adjoint pwd_set with the stored
// taps (reversed when forw), then the eps2 boundary terms; the float
// operations of predict_adj in its order.  tr (the chain's trace) and y (its
// scratch, holding the forward-substituted and then the solved trace) are
// interleaved, element k at k * yss; taps and fac point at the slope trace's
// column (element (e, k) at (e * n1 + k) * fss).  Operands are loaded in
// blocks of kAdjRows samples ahead of the arithmetic that uses them.
constexpr int kAdjRows = 8;
template <int NW>
__device__ void predict_adj_stored(int n1, float eps2, const float* __restrict__ taps,
                                   const float* __restrict__ fac, long fss, bool forw,
                                   float* __restrict__ tr, float* __restrict__ y, long yss) {
  constexpr int NA = 2 * NW + 1, NB = 2 * NW, R = kAdjRows;
  auto o_at = [&](int m, int k) { return fac[((long)m * n1 + k) * fss]; };
  // pass 1: y[i] = tr[i] - sum_{m < min(i, NB)} o[m][i-1-m] y[i-1-m]; rows
  // with fewer terms carry zero operands against the zero window
  {
    float Y[NB];
#pragma unroll
    for (int m = 0; m < NB; m++) Y[m] = 0.f;
    for (int i0 = 0; i0 < n1; i0 += R) {
      float t[R], ov[R][NB];
#pragma unroll
      for (int r = 0; r < R; r++) {
        const int i = i0 + r;
        t[r] = i < n1 ? tr[(long)i * yss] : 0.f;
#pragma unroll
        for (int m = 0; m < NB; m++) ov[r][m] = (i < n1 && i - 1 - m >= 0) ? o_at(m, i - 1 - m) : 0.f;
      }
#pragma unroll
      for (int r = 0; r < R; r++) {
        if (i0 + r < n1) {
          float v = t[r];
#pragma unroll
          for (int m = 0; m < NB; m++) v = __fsub_rn(v, __fmul_rn(ov[r][m], Y[m]));
#pragma unroll
          for (int m = NB - 1; m > 0; m--) Y[m] = Y[m - 1];
          Y[0] = v;
          y[(long)(i0 + r) * yss] = v;
        }
      }
    }
  }
  // pass 2: x[k] = y[k] / d[k] - sum_{m < min(n1-k-1, NB)} o[m][k] x[k+m+1]
  // (the stored o[m][k] are 0 beyond the band), in place in y
  {
    float X[NB];
#pragma unroll
    for (int m = 0; m < NB; m++) X[m] = 0.f;
    for (int j0 = 0; j0 < n1; j0 += R) {
      float t[R], dv[R], ov[R][NB];
#pragma unroll
      for (int r = 0; r < R; r++) {
        const int k = n1 - 1 - (j0 + r);
        t[r] = k >= 0 ? y[(long)k * yss] : 0.f;
        dv[r] = k >= 0 ? o_at(NB, k) : 1.f;
#pragma unroll
        for (int m = 0; m < NB; m++) ov[r][m] = k >= 0 ? o_at(m, k) : 0.f;
      }
#pragma unroll
      for (int r = 0; r < R; r++) {
        const int k = n1 - 1 - (j0 + r);
        if (k >= 0) {
          float v = __fdiv_rn(t[r], dv[r]);
#pragma unroll
          for (int m = 0; m < NB; m++) v = __fsub_rn(v, __fmul_rn(ov[r][m], X[m]));
#pragma unroll
          for (int m = NB - 1; m > 0; m--) X[m] = X[m - 1];
          X[0] = v;
          y[(long)k * yss] = v;
        }
      }
    }
  }
  const float b0 = y[0], b1 = y[yss], b2 = y[(long)(n1 - 2) * yss], b3 = y[(long)(n1 - 1) * yss];
  // pass 3: adjoint pwd_set.  tmp[k] = sum_{j=NA-1..0} a[j][k] x[k+NW-j]
  // (k in [NW, n1-NW)), then out[q] = sum_{j=NA-1..0} a[j][i] tmp[i] with
  // i = q+NW-j in [NW, n1-NW); both in the reference's accumulation order.
  FilterWin<NW> w;
  float tw[NA];
#pragma unroll
  for (int cc = 0; cc < NA; cc++) {
    tw[cc] = 0.f;
#pragma unroll
    for (int j = 0; j < NA; j++) w.a[cc][j] = 0.f;
  }
  auto column = [&](int cn, float* col) {
#pragma unroll
    for (int j = 0; j < NA; j++) col[j] = taps[((long)(forw ? NA - 1 - j : j) * n1 + cn) * fss];
  };
#pragma unroll
  for (int cc = 0; cc < NW; cc++)
    if (cc < n1) column(cc, w.a[NW + 1 + cc]);
  for (int q = 0; q < n1; q++) {
    const int cn = q + NW;
    shift_win<NW>(w);
#pragma unroll
    for (int cc = 0; cc < NA - 1; cc++) tw[cc] = tw[cc + 1];
    if (cn < n1)
      column(cn, w.a[2 * NW]);
    else
#pragma unroll
      for (int j = 0; j < NA; j++) w.a[2 * NW][j] = 0.f;
    float tk = 0.f;
    if (cn >= NW && cn < n1 - NW) {
#pragma unroll
      for (int j = NA - 1; j >= 0; j--) {
        const int ii = cn + NW - j;
        if (ii >= 0 && ii < n1) tk = __fadd_rn(tk, __fmul_rn(w.a[2 * NW][j], y[(long)ii * yss]));
      }
    }
    tw[NA - 1] = tk;
    float o = 0.f;
#pragma unroll
    for (int j = NA - 1; j >= 0; j--) {
      const int ii = q + NW - j;
      if (ii >= NW && ii < n1 - NW) o = __fadd_rn(o, __fmul_rn(w.a[2 * NW - j][j], tw[2 * NW - j]));
    }
    if (q == 0) o = __fadd_rn(o, __fmul_rn(eps2, b0));
    if (q == 1) o = __fadd_rn(o, __fmul_rn(eps2, b1));
    if (q == n1 - 2) o = __fadd_rn(o, __fmul_rn(eps2, b2));
    if (q == n1 - 1) o = __fadd_rn(o, __fmul_rn(eps2, b3));
    tr[(long)q * yss] = o;
  }
}

}  // namespace pwd
