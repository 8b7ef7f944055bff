// Table-driven FP64 exp and ln for the device kernels.
//
// GB300 issues FP64 at a small fraction of its FP32 rate, and CUDA's exp and
// log cost several times the instructions of these forms; both are used by
// the chemistry right-hand side and by the transport properties. The tables
// are built on the host by fill_exp_table / fill_log_table and live in each
// user's device buffer.
#pragma once

#include <cmath>

namespace edyn {

// 2^(j/64), j = 0..63: the table of texp.
inline void fill_exp_table(double* e2) {
  for (int j = 0; j < 64; ++j) e2[j] = (double)std::exp2((long double)j / 64.0L);
}

// ln(j/128) then 128/j for j = 90..181: the table of tlog (184 values).
inline void fill_log_table(double* lgt) {
  for (int j = 90; j < 182; ++j) {
    lgt[j - 90] = (double)std::log((long double)j / 128.0L);
    lgt[92 + j - 90] = (double)(128.0L / (long double)j);
  }
}

#ifdef __CUDACC__
// exp(x) in FP64 by the table-driven method of P. T. P. Tang (ACM TOMS 15,
// 1989): x = (64 m + j) ln2/64 + r with |r| <= ln2/128, so exp(x) =
// 2^m 2^(j/64) e^r, with 2^(j/64) from a 64-entry table (built on the host)
// and e^r - 1 from its degree-5 Taylor polynomial (truncation below 4e-17).
// About ten FP64 instructions, within 1 ulp of CUDA's exp. texp_r: arguments
// of a few units (no range handling); texp: x clamped to [-708, 709.7], so
// the result stays a normal number (exp(-708) stands in for anything smaller).
__device__ __forceinline__ double texp_r(double x, const double* e2) {
  const double magic = 6755399441055744.0;  // 1.5 * 2^52: rounds to an integer
  const double k64 = 92.33248261689366;     // 64 / ln 2
  const double l1 = 0.010830424695086549;   // ln2/64, leading bits (low 20 bits zero)
  const double l2 = 1.162596423439437e-12;  // ln2/64 - l1
  const double tk = fma(x, k64, magic);
  const double kd = tk - magic;
  const int ki = __double2loint(tk);
  double r = fma(-kd, l1, x);
  r = fma(-kd, l2, r);
  double s = fma(r, 1.0 / 120.0, 1.0 / 24.0);
  s = fma(s, r, 1.0 / 6.0);
  s = fma(s, r, 0.5);
  const double p = fma(r * r, s, r);
  const double tj = e2[ki & 63];
  const double v = fma(tj, p, tj);
  return __hiloint2double(__double2hiint(v) + ((ki >> 6) << 20), __double2loint(v));
}
__device__ __forceinline__ double texp(double x, const double* e2) {
  return texp_r(fmin(fmax(x, -708.0), 709.7), e2);
}
// texp for arguments of magnitude below 1e13 (Arrhenius, fall-off): the
// range is clamped on the integer pipe instead of by two FP64 min/max
// (206 cycles each on GB300); beyond [-708, 709.7] it returns the
// bound's value, exp(-708) standing in for anything smaller.
__device__ __forceinline__ double texp_a(double x, const double* e2) {
  const double magic = 6755399441055744.0;
  const double k64 = 92.33248261689366;
  const double l1 = 0.010830424695086549;
  const double l2 = 1.162596423439437e-12;
  const double tk = fma(x, k64, magic);
  const double kd = tk - magic;
  double r = fma(-kd, l1, x);
  r = fma(-kd, l2, r);
  double s = fma(r, 1.0 / 120.0, 1.0 / 24.0);
  s = fma(s, r, 1.0 / 6.0);
  s = fma(s, r, 0.5);
  const double p = fma(r * r, s, r);
  // 64 m + j, kept where 2^m (1 + p) 2^(j/64) stays a normal number
  const int ki = min(max(__double2loint(tk), -65344), 65471);
  const double tj = e2[ki & 63];
  const double v = fma(tj, p, tj);
  return __hiloint2double(__double2hiint(v) + ((ki >> 6) << 20), __double2loint(v));
}

// ln(x) in FP64 for normal x > 0, table-driven: x = 2^m f with f in
// [sqrt(1/2), sqrt(2)), F = j/128 the grid point nearest f (j in [90, 181]),
// r = (f - F)/F with |r| <= 0.0056; f - F is exact and 1/F comes from the
// table. ln x = m ln2 + ln F + log1p(r), log1p from its series to r^7
// (truncation below 2e-19). Near x = 1, F = 1 and ln x = log1p(r) without
// cancellation; elsewhere |ln F| or |m ln2| dominates the sum. About a dozen
// FP64 instructions against ~2,000 cycles for CUDA's log on GB300.
__device__ __forceinline__ double tlog(double x, const double* lg) {
  const double ln2_hi = 0.6931467056274414;   // ln 2, low 32 bits zero: m ln2_hi is exact
  const double ln2_lo = 4.7493250390316726e-07; // ln 2 - ln2_hi
  const int hi = __double2hiint(x), lo = __double2loint(x);
  const int mant = hi & 0xfffff;
  int m = ((hi >> 20) & 0x7ff) - 1023;
  int j, fe;
  if (mant < 0x6a09e) {  // f = 1.mant < sqrt 2
    j = 128 + ((mant + (1 << 12)) >> 13);
    fe = 0x3ff00000;
  } else {               // use f/2 in [sqrt(1/2), 1)
    j = 64 + ((mant + (1 << 13)) >> 14);
    fe = 0x3fe00000;
    m += 1;
  }
  const double f = __hiloint2double(mant | fe, lo);
  const double r = (f - j * 0.0078125) * lg[92 + j - 90];
  double s = fma(r, 1.0 / 7.0, -1.0 / 6.0);
  s = fma(s, r, 0.2);
  s = fma(s, r, -0.25);
  s = fma(s, r, 1.0 / 3.0);
  s = fma(s, r, -0.5);
  const double p = fma(r * r, s, r);
  // (double)m from its bits: 2^52 + 2^31 + m, minus the offset
  const double md = __hiloint2double(0x43300000, m ^ 0x80000000) - 4503601774854144.0;
  return fma(md, ln2_hi, lg[j - 90]) + fma(md, ln2_lo, p);
}


#endif  // __CUDACC__

}  // namespace edyn
