// CH4 + OH potential (Espinosa-Garcia, Corchado, J. Chem. Phys. 112, 5731
// (2000)) as GB300 device code: a drop-in for Caracal's egrad_ch4oh
// (src/egrad_ch4oh.f:69-124) with its POTLIB wrapper in Caracal's settings
// (bohr/Hartree user units, no relabelling: the routines of
// src/util_ch4oh.f are identities).  The same code with the constants of
// src/egrad_geh4oh.f is the GeH4 + OH surface (egrad_geh4oh :33-67): its
// routines differ from CH4 + OH's only in the pyramid angle of refangles and
// the uncut sphi of switchf (ParCH4OH / ParGeH4OH below).
//
// One thread evaluates one bead.  Routines restated (src/egrad_ch4oh.f):
// POT_ch4oh :157, coorden :288, refangles :374, stretch :517, opbend :782,
// ipbend :938, calcdelta :1177, opforce :1435, ipforce :1549, switchf :1748;
// constants from BLOCK DATA PTPACM_ch4oh :2007 with PREPOT_ch4oh's unit
// factors (all REAL(8)).  Atoms: 0 H(methane, nnh(4)), 1 C (nnc), 2,3,4
// H(methane, nnh(1..3)), 5 O (nnb), 6 H of OH (nno); methane H i = 0..3 are
// atoms {2,3,4,0}.
//
// The surface is the CH4 + H one (same functional forms, own constants and
// the original POTLIB switching constants) plus an O-H Morse stretch and four
// H(i)-O-H(O) harmonic bends with a tanh-switched force constant.  The
// switched C-B triplet depth d3cb(rav) of stretch_ch4oh has amplitude
// a3cb = 0, so d3cb = d3cbi and its derivative terms vanish; they are folded
// away at compile time.  GPU restructuring as for CH4 + H (unrolled loops,
// shared reciprocals, the opbend k <-> l swap as a sign); the energy and
// gradient unit factors 0.03812 and 0.0201723 are the reference's.
//
// Mixed form (F = float): as for CH4 + H, positions enter as float pairs
// (ff32.cuh), the LEPS stretch block -- whose Q and exchange derivatives are
// large and cancel near the bond minima -- and the in-plane bends' angle
// differences from their references are formed in float-pair arithmetic,
// and the stretch gradient is summed as float pairs; the rest is FP32.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

#include "ff32.cuh"

namespace cr {
namespace ch4oh {

// The constants of BLOCK DATA PTPACM_ch4oh (src/egrad_ch4oh.f:2064-2106) and
// PTPACM_geh4oh (src/egrad_geh4oh.f:2001-2045) after PREPOT's / initialize's
// conversions (src/egrad_ch4oh.f:1987-2003): d's * 0.041840, force constants
// * 6.022045, anh2oeq * 2 pi / 360.  The two surfaces share these:
constexpr double r0hh = 0.97060;
constexpr double a3cb = 0.000000 * 0.041840, b3cb = 0.900000, rcbsp = 2.606485;
constexpr double aphi = 0.5287900, bphi = 0.4006600;
constexpr double atheta = 0.9078700, btheta = 0.3548900, ctheta = 1.8915500;
constexpr double hch3 = 0.1915000 * 6.022045, ak = 0.1260000 * 6.022045;
constexpr double aa2 = 1.599960, aa4 = 11.569980;
constexpr double fkh2oeq = 0.7300000 * 6.022045, alph2o = 1.1080000;
constexpr double anh2oeq = 104.7132000 * (2.0 * 3.141592653589793 / 360.0);
static_assert(a3cb == 0.0, "the d3cb(rav) switch is folded away for a3cb = 0");
// switchf local constants (the original POTLIB values)
constexpr double a1s = 1.5313681e-7, b1s = -4.6696246, a2s = 1.0147402e-7, b2s = -12.363798;

// The constants that differ.  tau_py is the pyramid angle of refangles'
// sphi term (pi/2: planar CH3; 0.678 pi: pyramidal GeH3,
// src/egrad_geh4oh.f:368-392); sphi_cut keeps switchf's rch < 3.8 condition
// on sphi (CH4 + OH; GeH4 + OH evaluates sphi at every distance,
// src/egrad_geh4oh.f:1792-1804).
struct ParCH4OH {
  static constexpr double r0ch = 1.09397, a1ch = 1.78000, b1ch = 0.15000, c1ch = 15.00000;
  static constexpr double ahh = 2.15000, r0cb = 1.49092, acb = 2.98688;
  static constexpr double d1ch = 112.17000 * 0.041840, d3ch = 32.65328 * 0.041840;
  static constexpr double d1hh = 125.44000 * 0.041840, d3hh = 20.41017 * 0.041840;
  static constexpr double d1cb = 91.47526 * 0.041840, d3cbi = 112.69509 * 0.041840;
  static constexpr double a3s = 0.1419100, b3s = -0.3068400, cphi = 1.9209900;
  static constexpr double fch3 = 0.0740000 * 6.022045, fkinf = 0.4400000 * 6.022045;
  static constexpr double aa1 = 0.303746, aa3 = 3.216595;
  static constexpr double tau_py = 0.5 * 3.141592653589793;
  static constexpr bool sphi_cut = true;
};
struct ParGeH4OH {
  static constexpr double r0ch = 1.52500, a1ch = 1.43925, b1ch = 0.12330, c1ch = 2.00400;
  static constexpr double ahh = 2.18200, r0cb = 1.90035, acb = 0.67621;
  static constexpr double d1ch = 86.50000 * 0.041840, d3ch = 41.50000 * 0.041840;
  static constexpr double d1hh = 120.94800 * 0.041840, d3hh = 31.86417 * 0.041840;
  static constexpr double d1cb = 41.50283 * 0.041840, d3cbi = 10.50589 * 0.041840;
  static constexpr double a3s = 0.2019100, b3s = -0.6068400, cphi = 11.8809900;
  static constexpr double fch3 = 0.0150000 * 6.022045, fkinf = 0.3060000 * 6.022045;
  static constexpr double aa1 = 0.173746, aa3 = 2.166595;
  static constexpr double tau_py = 0.678 * 3.141592653589793;
  static constexpr bool sphi_cut = false;
};

template <class F> __device__ inline F t_exp(F x);
template <> __device__ inline double t_exp<double>(double x) { return exp(x); }
template <> __device__ inline float t_exp<float>(float x) { return expf(x); }
template <class F> __device__ inline F t_sqrt(F x);
template <> __device__ inline double t_sqrt<double>(double x) { return sqrt(x); }
template <> __device__ inline float t_sqrt<float>(float x) { return sqrtf(x); }
template <class F> __device__ inline F t_acos(F x);
template <> __device__ inline double t_acos<double>(double x) { return acos(x); }
template <> __device__ inline float t_acos<float>(float x) { return acosf(x); }
template <class F> __device__ inline F t_tanh(F x);
template <> __device__ inline double t_tanh<double>(double x) { return tanh(x); }
template <> __device__ inline float t_tanh<float>(float x) { return tanhf(x); }
template <class F> __device__ inline F t_cosh(F x);
template <> __device__ inline double t_cosh<double>(double x) { return cosh(x); }
template <> __device__ inline float t_cosh<float>(float x) { return coshf(x); }

// methane H i (0..3, nnh order) -> atom index
__device__ constexpr int NH(int i) { return i == 0 ? 2 : i == 1 ? 3 : i == 2 ? 4 : 0; }
constexpr int NC = 1, NB = 5, NO = 6;

template <class F>
struct Geo {
  F tcb[3], tno[3], tch[4][3], tbh[4][3];
  F rcb, rno, rch[4], rbh[4], ircb, irno, irch[4], irbh[4];
  F uch[4][3];  // tch / rch
};

// 1 - tanh(arg) and its derivative factor -1/cosh(arg)^2, with Caracal's
// tanh(19) = 1 cutoff (switchf_ch4oh)
template <class F>
__device__ inline void switch_fn(F arg, F darg_num, F& s, F& ds) {
  if (arg < F(19.0)) {
    s = F(1) - t_tanh<F>(arg);
    F ch = t_cosh<F>(arg);
    ds = -darg_num / (ch * ch);
  } else {
    s = F(0);
    ds = F(0);
  }
}

template <class F, class K>
__device__ inline void egrad(const double (&qb)[21], double& Vout, double (&gout)[21]) {
  constexpr double r0ch = K::r0ch, a1ch = K::a1ch, b1ch = K::b1ch, c1ch = K::c1ch;
  constexpr double ahh = K::ahh, r0cb = K::r0cb, acb = K::acb;
  constexpr double d1ch = K::d1ch, d3ch = K::d3ch, d1hh = K::d1hh, d3hh = K::d3hh;
  constexpr double d1cb = K::d1cb, d3cb = K::d3cbi - a3cb;
  constexpr double a3s = K::a3s, b3s = K::b3s, cphi = K::cphi;
  constexpr double fch3 = K::fch3, fkinf = K::fkinf, aa1 = K::aa1, aa3 = K::aa3;
  // ---- positions in Angstrom (POT_ch4oh: q = R * 0.52918) and coorden
  double qa[21];
#pragma unroll
  for (int x = 0; x < 21; ++x) qa[x] = qb[x] * 0.52918;
  Geo<F> G;
  constexpr bool kPair = std::is_same<F, float>::value;
  ff Xtcb[3], Xtno[3], Xtch[4][3], Xtbh[4][3], Xrch[4];
  if constexpr (kPair) {
    ff X[21];
#pragma unroll
    for (int x = 0; x < 21; ++x) {
      const float h = __double2float_rn(qa[x]);
      X[x] = ff{h, __double2float_rn(qa[x] - (double)h)};
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      Xtcb[d] = X[3 * NC + d] - X[3 * NB + d];
      G.tcb[d] = ff_float(Xtcb[d]);
      Xtno[d] = X[3 * NO + d] - X[3 * NB + d];
      G.tno[d] = ff_float(Xtno[d]);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        Xtch[i][d] = X[3 * NC + d] - X[3 * NH(i) + d];
        Xtbh[i][d] = X[3 * NB + d] - X[3 * NH(i) + d];
        G.tch[i][d] = ff_float(Xtch[i][d]);
        G.tbh[i][d] = ff_float(Xtbh[i][d]);
      }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
      Xrch[i] = ff_sqrt(Xtch[i][0] * Xtch[i][0] + Xtch[i][1] * Xtch[i][1] + Xtch[i][2] * Xtch[i][2]);
  } else {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      G.tcb[d] = (F)(qa[3 * NC + d] - qa[3 * NB + d]);
      G.tno[d] = (F)(qa[3 * NO + d] - qa[3 * NB + d]);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        G.tch[i][d] = (F)(qa[3 * NC + d] - qa[3 * NH(i) + d]);
        G.tbh[i][d] = (F)(qa[3 * NB + d] - qa[3 * NH(i) + d]);
      }
    }
  }
  G.rcb = t_sqrt<F>(G.tcb[0] * G.tcb[0] + G.tcb[1] * G.tcb[1] + G.tcb[2] * G.tcb[2]);
  G.ircb = F(1) / G.rcb;
  G.rno = t_sqrt<F>(G.tno[0] * G.tno[0] + G.tno[1] * G.tno[1] + G.tno[2] * G.tno[2]);
  G.irno = F(1) / G.rno;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    G.rch[i] = t_sqrt<F>(G.tch[i][0] * G.tch[i][0] + G.tch[i][1] * G.tch[i][1] + G.tch[i][2] * G.tch[i][2]);
    G.rbh[i] = t_sqrt<F>(G.tbh[i][0] * G.tbh[i][0] + G.tbh[i][1] * G.tbh[i][1] + G.tbh[i][2] * G.tbh[i][2]);
    G.irch[i] = F(1) / G.rch[i];
    G.irbh[i] = F(1) / G.rbh[i];
#pragma unroll
    for (int d = 0; d < 3; ++d) G.uch[i][d] = G.tch[i][d] * G.irch[i];
  }
  F pdot[21];
#pragma unroll
  for (int x = 0; x < 21; ++x) pdot[x] = F(0);
  // mixed form: the stretch gradient, summed as float pairs (its terms are
  // large and cancel on each atom); the other terms add into pdot in FP32
  ff psx[kPair ? 21 : 1];
#pragma unroll
  for (int x = 0; x < (kPair ? 21 : 1); ++x) psx[x] = ff{0.f, 0.f};

  // ---- switching functions (switchf_ch4oh)
  F s1[4], ds1[4], s2[4], ds2[4], s3[4], ds3[4], sphi[4], dsphi[4], sth[4], dsth[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const F r = G.rch[i], x = r - F(r0ch);
    F y1 = r - F(b1s), y1_2 = y1 * y1, y1_4 = y1_2 * y1_2, y1_7 = y1_4 * y1_2 * y1, y1_8 = y1_4 * y1_4;
    switch_fn<F>(F(a1s) * x * y1_8, F(a1s) * (y1_8 + F(8) * x * y1_7), s1[i], ds1[i]);
    F y2 = r - F(b2s), y2_2 = y2 * y2, y2_4 = y2_2 * y2_2, y2_5 = y2_4 * y2, y2_6 = y2_4 * y2_2;
    switch_fn<F>(F(a2s) * x * y2_6, F(a2s) * (y2_6 + F(6) * x * y2_5), s2[i], ds2[i]);
    F y3 = r - F(b3s);
    switch_fn<F>(F(a3s) * x * (y3 * y3),
                 F(a3s) * (F(3) * r * r - F(2) * r * F(r0ch + 2.0 * b3s) + F(b3s * (b3s + 2.0 * r0ch))),
                 s3[i], ds3[i]);
    sphi[i] = F(0);
    dsphi[i] = F(0);
    if (!K::sphi_cut || r < F(3.8)) {
      F xc = r - F(cphi);
      F e = t_exp<F>(F(bphi) * xc * xc * xc);
      F arg = F(aphi) * x * e;
      // FP32 only: past arg = 19, 1 - tanh is 0 in float and exp or cosh
      // overflows first (GeH4 + OH, r > 17.9 A); FP64 follows the reference
      if (!kPair || arg < F(19.0)) {
        F ch = t_cosh<F>(arg);
        sphi[i] = F(1) - t_tanh<F>(arg);
        dsphi[i] = -(F(aphi) * (F(1) + F(3) * F(bphi) * x * xc * xc) * e) / (ch * ch);
      }
    }
    if (r < F(3.8)) {
      F xt = r - F(ctheta);
      F et = t_exp<F>(F(btheta) * xt * xt * xt);
      F argt = F(atheta) * x * et;
      F cht = t_cosh<F>(argt);
      sth[i] = F(1) - t_tanh<F>(argt);
      dsth[i] = -(F(atheta) * (F(1) + F(3) * F(btheta) * x * xt * xt) * et) / (cht * cht);
    } else {
      sth[i] = F(0);
      dsth[i] = F(0);
    }
  }

  // ---- reference angles (refangles_ch4oh): theta0[i][j], dtheta0[i][j][k]
  const double tau = 1.9106332362490186;  // acos(-1/3)
  const double pi = 3.141592653589793;
  const F A = F(tau - K::tau_py), B = F(tau - 2.0 * pi / 3.0);
  F th0[4][4], dth0[4][4][4];
  F th0m[4][4];  // th0 - tau, without the rounding of tau (the mixed form's bend differences)
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      th0[i][j] = F(0);
      th0m[i][j] = F(0);
#pragma unroll
      for (int k = 0; k < 4; ++k) dth0[i][j][k] = F(0);
    }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i + 1; j < 4; ++j) {
      // the two H not in the pair
      int m = -1, n = -1;
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (k != i && k != j) {
          if (m < 0) m = k;
          else n = k;
        }
      const F tm = A * (sphi[i] * sphi[j] - F(1)) + B * (sth[m] * sth[n] - F(1));
      F t = F(tau) + tm;
      th0[i][j] = t;
      th0[j][i] = t;
      th0m[i][j] = tm;
      th0m[j][i] = tm;
      F di = A * dsphi[i] * sphi[j], dj = A * sphi[i] * dsphi[j];
      F dm = B * dsth[m] * sth[n], dn = B * sth[m] * dsth[n];
      dth0[i][j][i] = di; dth0[j][i][i] = di;
      dth0[i][j][j] = dj; dth0[j][i][j] = dj;
      dth0[i][j][m] = dm; dth0[j][i][m] = dm;
      dth0[i][j][n] = dn; dth0[j][i][n] = dn;
    }

  // ---- stretching (stretch_ch4oh)
  F vstr = F(0);
  if constexpr (kPair) {
    // Mixed form.  Per C-H bond i the LEPS gradient collapses onto three
    // scalars: T_i (along the C-H_i stretch, Q and exchange terms together),
    // U_i (C-O) and W_i (O-H_i), formed in float-pair arithmetic and rounded
    // once; the vectors they multiply are float pairs too.
    const F rav = (G.rch[0] + G.rch[1] + G.rch[2] + G.rch[3]) * F(0.25);
    const F arga = F(c1ch) * (rav - F(r0ch));
    F dumach;
    if (arga < F(19.0)) {
      const F ch = t_cosh<F>(arga);
      dumach = F(b1ch * c1ch) / (F(2) * (ch * ch));
    } else {
      dumach = F(0);
    }
    constexpr ff D1ch = ff_const(d1ch), D3ch = ff_const(d3ch), D1hh = ff_const(d1hh), D3hh = ff_const(d3hh);
    constexpr ff D1cb = ff_const(d1cb), D3cb = ff_const(d3cb);
    constexpr ff Sqch = ff_const(d1ch + d3ch), Dfch = ff_const(d1ch - d3ch);
    constexpr ff Sqhh = ff_const(d1hh + d3hh), Dfhh = ff_const(d1hh - d3hh);
    constexpr ff Sqcb = ff_const(d1cb + d3cb), Dfcb = ff_const(d1cb - d3cb);
    constexpr ff R0ch = ff_const(r0ch), R0hh = ff_const(r0hh), R0cb = ff_const(r0cb);
    constexpr ff Acb = ff_const(acb), Ahh = ff_const(ahh);
    auto norm3 = [](const ff (&v)[3]) { return ff_sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
    const ff rcb = norm3(Xtcb);
    const ff ecb1 = ff_exp(-(Acb * (rcb - R0cb))), ecb2 = ecb1 * ecb1;
    const ff vqcb = (D1cb * (ecb2 - ecb1 * 2.f) + D3cb * (ecb2 + ecb1 * 2.f)) * 0.5f;
    const ff vjcb = (D1cb * (ecb2 - ecb1 * 2.f) - D3cb * (ecb2 + ecb1 * 2.f)) * 0.5f;
    const ff dqcb = -(Acb * (Sqcb * ecb2 - Dfcb * ecb1));  // d vqcb / d rcb
    const ff djcb = -(Acb * (Dfcb * ecb2 - Sqcb * ecb1));  // d vjcb / d rcb
    // ach = a1 + b1 (tanh(arga) + 1) / 2 = a1 + b1 / (1 + exp(-2 arga))
    ff achx = ff_const(a1ch + b1ch);
    if (arga < F(19.0)) {
      constexpr ff A1 = ff_const(a1ch), B1 = ff_const(b1ch), C1 = ff_const(c1ch);
      const ff ravx = (Xrch[0] + Xrch[1] + Xrch[2] + Xrch[3]) * 0.25f;
      const ff e2 = ff_exp(-(C1 * (ravx - R0ch)) * 2.f);
      achx = A1 + B1 / (ff_from(1.f) + e2);
    }
    ff vsum = ff_from(0.f);
    F achdc[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) achdc[d] = dumach * (G.uch[0][d] + G.uch[1][d] + G.uch[2][d] + G.uch[3][d]) * F(0.25);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const ff rch = Xrch[i], rbh = norm3(Xtbh[i]);
      const ff xch = rch - R0ch;
      const ff ec1 = ff_exp(-(achx * xch)), ec2 = ec1 * ec1;
      const ff vqch = (D1ch * (ec2 - ec1 * 2.f) + D3ch * (ec2 + ec1 * 2.f)) * 0.5f;
      const ff vjch = (D1ch * (ec2 - ec1 * 2.f) - D3ch * (ec2 + ec1 * 2.f)) * 0.5f;
      const ff eh1 = ff_exp(-(Ahh * (rbh - R0hh))), eh2 = eh1 * eh1;
      const ff vqbh = (D1hh * (eh2 - eh1 * 2.f) + D3hh * (eh2 + eh1 * 2.f)) * 0.5f;
      const ff vjbh = (D1hh * (eh2 - eh1 * 2.f) - D3hh * (eh2 + eh1 * 2.f)) * 0.5f;
      const ff e12 = vjch - vjcb, e23 = vjcb - vjbh, e31 = vjbh - vjch;
      const ff vj = -ff_sqrt((e12 * e12 + e23 * e23 + e31 * e31) * 0.5f);
      vsum += vqch + vqcb + vqbh + vj;
      const ff factj = ff_recip(vj) * 0.5f;
      const ff brq = Sqch * ec2 - Dfch * ec1, brj = Dfch * ec2 - Sqch * ec1;
      const ff dqbh = -(Ahh * (Sqhh * eh2 - Dfhh * eh1)), djbh = -(Ahh * (Dfhh * eh2 - Sqhh * eh1));
      // T: -(d V / d (ach * xch)); U: d V / d rcb (per unit rcb); W: d V / d rbh
      const ff T = brq + (e12 - e31) * factj * brj;
      const ff U = (-dqcb + (e12 - e23) * factj * djcb) / rcb;
      const ff W = (dqbh + (e31 - e23) * factj * djbh) / rbh;
      const ff irch = ff_recip(rch);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const ff u = Xtch[i][d] * irch;
        const ff tcb = Xtcb[d], tbh = Xtbh[i][d];
        const ff gc = achx * u + xch * achdc[d];
        const ff gh = achx * u + xch * (dumach * G.uch[i][d] * F(0.25));
        psx[3 * NC + d] -= gc * T + tcb * U;
        psx[3 * NH(i) + d] += gh * T - tbh * W;
        psx[3 * NB + d] += tcb * U + tbh * W;
        const ff xT = xch * T;
#pragma unroll
        for (int k = 1; k <= 3; ++k) {
          const int j = (i + k) & 3;
          psx[3 * NH(j) + d] += xT * (dumach * G.uch[j][d] * F(0.25));
        }
      }
    }
    // O-H Morse stretch (stretch_ch4oh :602-605, :620-632, :711-716), its
    // 1 - exp(-a (r - r0)) near the minimum in float pairs too
    const ff rno = norm3(Xtno);
    const ff eoh = ff_exp(-(Ahh * (rno - R0hh)));
    const ff omo = ff_from(1.f) - eoh;
    vsum += D1hh * (omo * omo);
    const ff de = (ff_const(2.0 * ahh * d1hh) * omo * eoh) / rno;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      psx[3 * NB + d] -= de * Xtno[d];
      psx[3 * NO + d] += de * Xtno[d];
    }
    vstr = ff_float(vsum);
  } else
  {
    F rav = (G.rch[0] + G.rch[1] + G.rch[2] + G.rch[3]) * F(0.25);
    F arga = F(c1ch) * (rav - F(r0ch));
    F ach, dumach;
    if (arga < F(19.0)) {
      ach = F(a1ch) + F(b1ch) * (t_tanh<F>(arga) + F(1)) * F(0.5);
      F ch = t_cosh<F>(arga);
      dumach = F(b1ch * c1ch) / (F(2) * (ch * ch));
    } else {
      ach = F(a1ch + b1ch);
      dumach = F(0);
    }
    F ecb2 = t_exp<F>(F(-2.0 * acb) * (G.rcb - F(r0cb))), ecb1 = t_exp<F>(F(-acb) * (G.rcb - F(r0cb)));
    F vqcb = (F(d1cb) * (ecb2 - F(2) * ecb1) + F(d3cb) * (ecb2 + F(2) * ecb1)) * F(0.5);
    F vjcb = (F(d1cb) * (ecb2 - F(2) * ecb1) - F(d3cb) * (ecb2 + F(2) * ecb1)) * F(0.5);
    F dumqcb = F(-acb) * (F(d1cb + d3cb) * ecb2 - F(d1cb - d3cb) * ecb1) * G.ircb;
    F jcb_num = F(-acb) * (F(d1cb - d3cb) * ecb2 - F(d1cb + d3cb) * ecb1) * G.ircb;
    F achdc[3] = {F(0), F(0), F(0)};
#pragma unroll
    for (int d = 0; d < 3; ++d)
      achdc[d] = dumach * (G.uch[0][d] + G.uch[1][d] + G.uch[2][d] + G.uch[3][d]) * F(0.25);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const F xch = G.rch[i] - F(r0ch);
      F ec2 = t_exp<F>(F(-2) * ach * xch), ec1 = t_exp<F>(-ach * xch);
      F vqch = (F(d1ch) * (ec2 - F(2) * ec1) + F(d3ch) * (ec2 + F(2) * ec1)) * F(0.5);
      F vjch = (F(d1ch) * (ec2 - F(2) * ec1) - F(d3ch) * (ec2 + F(2) * ec1)) * F(0.5);
      F eh2 = t_exp<F>(F(-2.0 * ahh) * (G.rbh[i] - F(r0hh))), eh1 = t_exp<F>(F(-ahh) * (G.rbh[i] - F(r0hh)));
      F vqbh = (F(d1hh) * (eh2 - F(2) * eh1) + F(d3hh) * (eh2 + F(2) * eh1)) * F(0.5);
      F vjbh = (F(d1hh) * (eh2 - F(2) * eh1) - F(d3hh) * (eh2 + F(2) * eh1)) * F(0.5);
      F e12 = vjch - vjcb, e23 = vjcb - vjbh, e31 = vjbh - vjch;
      F vj = -t_sqrt<F>((e12 * e12 + e23 * e23 + e31 * e31) * F(0.5));
      vstr += vqch + vqcb + vqbh + vj;
      F dumqbh = F(-ahh) * (F(d1hh + d3hh) * eh2 - F(d1hh - d3hh) * eh1) * G.irbh[i];
      F factj = F(0.5) / vj;
      F dumjcb = jcb_num * factj;
      F dumjbh = F(-ahh) * (F(d1hh - d3hh) * eh2 - F(d1hh + d3hh) * eh1) * factj * G.irbh[i];
      F brq = F(d1ch + d3ch) * ec2 - F(d1ch - d3ch) * ec1;
      F brj = (F(d1ch - d3ch) * ec2 - F(d1ch + d3ch) * ec1) * factj;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const F tcb = G.tcb[d], tbh = G.tbh[i][d];
        pdot[3 * NB + d] += -tcb * dumqcb + tbh * dumqbh + e12 * (dumjcb * tcb) +
                            e23 * (-dumjcb * tcb - dumjbh * tbh) + e31 * dumjbh * tbh;
        const F achdh_i = -dumach * G.uch[i][d] * F(0.25);
        const F gc = ach * G.uch[i][d] + achdc[d] * xch;   // -(d a/d c) factor
        const F gh = ach * G.uch[i][d] - achdh_i * xch;    //  (d a/d h_i) factor
        const F dumjch = -gc * brj;
        const F dumjhi = gh * brj;
        pdot[3 * NC + d] += -gc * brq + tcb * dumqcb + e12 * (dumjch - dumjcb * tcb) + e23 * dumjcb * tcb - e31 * dumjch;
        pdot[3 * NH(i) + d] += gh * brq - tbh * dumqbh + e12 * dumjhi + e23 * dumjbh * tbh + e31 * (-dumjbh * tbh - dumjhi);
#pragma unroll
        for (int k = 1; k <= 3; ++k) {
          const int j = (i + k) & 3;
          const F achdh_j = -dumach * G.uch[j][d] * F(0.25);
          const F c = -achdh_j * xch;
          pdot[3 * NH(j) + d] += c * brq + (e12 - e31) * (c * brj);
        }
      }
    }
    // O-H Morse stretch (stretch_ch4oh :602-605, :620-632, :711-716)
    const F eoh = t_exp<F>(F(-ahh) * (G.rno - F(r0hh)));
    const F omo = F(1) - eoh;
    vstr += F(d1hh) * (omo * omo);
    const F de = F(2.0 * ahh * d1hh) * omo * eoh * G.irno;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      pdot[3 * NB + d] -= de * G.tno[d];
      pdot[3 * NO + d] += de * G.tno[d];
    }
  }

  // ---- out-of-plane bends (opbend_ch4oh, opforce_ch4oh, calcdelta_ch4oh)
  F vop = F(0);
  {
    F sw[4], dsw[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      F prod = F(1);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (k != i) prod *= s3[k];
      sw[i] = (F(1) - s3[i]) * prod;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (k == i) {
          dsw[i][k] = -ds3[i] * prod;
        } else {
          F pr = F(1);
#pragma unroll
          for (int m = 0; m < 4; ++m)
            if (m != i && m != k) pr *= s3[m];
          dsw[i][k] = (F(1) - s3[i]) * ds3[k] * pr;
        }
      }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int j = (i + 1) & 3, k = (i + 2) & 3, l = (i + 3) & 3;
      const int in3[3] = {j, k, l};
      F a[3], b[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        a[d] = (F)(qa[3 * NH(k) + d] - qa[3 * NH(j) + d]);
        b[d] = (F)(qa[3 * NH(l) + d] - qa[3 * NH(j) + d]);
      }
      F axb[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
      F norma = t_sqrt<F>(axb[0] * axb[0] + axb[1] * axb[1] + axb[2] * axb[2]);
      F inorm = F(1) / norma;
      // cumulative swap of k and l for each positive (a x b).c (src/egrad_ch4oh.f, opbend)
      bool flip = false;
#pragma unroll
      for (int ii = 0; ii < 3; ++ii) {
        const int m = in3[ii];
        F argd = -(axb[0] * G.uch[m][0] + axb[1] * G.uch[m][1] + axb[2] * G.uch[m][2]) * inorm;
        if (argd > F(0)) flip = !flip;
      }
      const F s = flip ? F(-1) : F(1);
#pragma unroll
      for (int d = 0; d < 3; ++d) axb[d] *= s;
      // daxb[pos][ind][comp]: derivative of a x b wrt atom in3[pos], coordinate ind
      F dax[3][3][3];
      const F bma[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
      const F* vv[3] = {bma, b, a};
      const F sg[3] = {F(1), F(-1), F(1)};
#pragma unroll
      for (int pos = 0; pos < 3; ++pos) {
        const F* w = vv[pos];
        const F g = sg[pos] * s;
        dax[pos][0][0] = F(0);        dax[pos][0][1] = g * w[2];   dax[pos][0][2] = -g * w[1];
        dax[pos][1][0] = -g * w[2];   dax[pos][1][1] = F(0);       dax[pos][1][2] = g * w[0];
        dax[pos][2][0] = g * w[1];    dax[pos][2][1] = -g * w[0];  dax[pos][2][2] = F(0);
      }
      F delta[3], argd[3], c[3][3];
      F sum2 = F(0), sum4 = F(0);
#pragma unroll
      for (int ii = 0; ii < 3; ++ii) {
        const int m = in3[ii];
#pragma unroll
        for (int d = 0; d < 3; ++d) c[ii][d] = -G.uch[m][d];
        argd[ii] = (axb[0] * c[ii][0] + axb[1] * c[ii][1] + axb[2] * c[ii][2]) * inorm;
        delta[ii] = t_acos<F>(argd[ii]) - th0[i][m];
        F d2 = delta[ii] * delta[ii];
        sum2 += d2;
        sum4 += d2 * d2;
      }
      const F fd = F(fch3) * sw[i], hd = F(hch3) * sw[i];
      vop += fd * sum2 + hd * sum4;
      const F inorm3 = inorm * inorm * inorm;
#pragma unroll
      for (int ii = 0; ii < 3; ++ii) {
        const int m = in3[ii];
        const F coef = F(2) * fd * delta[ii] + F(4) * hd * delta[ii] * delta[ii] * delta[ii];
        const F irs = F(1) / t_sqrt<F>(F(1) - argd[ii] * argd[ii]);
#pragma unroll
        for (int ind = 0; ind < 3; ++ind) {
          const F d0 = dth0[i][m][i] * G.uch[i][ind];   // deldot wrt h_i
          pdot[3 * NH(i) + ind] += coef * d0;
          pdot[3 * NC + ind] -= coef * d0;
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) {
            const int mj = in3[jj];
            F at1 = (axb[0] * dax[jj][ind][0] + axb[1] * dax[jj][ind][1] + axb[2] * dax[jj][ind][2]) * inorm3;
            F at3 = (dax[jj][ind][0] * inorm - at1 * axb[0]) * c[ii][0] +
                    (dax[jj][ind][1] * inorm - at1 * axb[1]) * c[ii][1] +
                    (dax[jj][ind][2] * inorm - at1 * axb[2]) * c[ii][2];
            F at4 = F(0);
            if (ii == jj) {
              // axb . cdot(m, :, ind), cdot = d c / d h_m
              const F ir = G.irch[m];
              F dot = F(0);
#pragma unroll
              for (int cc = 0; cc < 3; ++cc) {
                F cd = G.tch[m][ind] * c[ii][cc] * ir * ir;
                if (cc == ind) cd += ir;
                dot += axb[cc] * cd;
              }
              at4 = dot * inorm;
            }
            const F at5 = dth0[i][m][mj] * G.uch[mj][ind];
            F dd = -irs * (at3 + at4) + at5;
            pdot[3 * NH(mj) + ind] += coef * dd;
            dd = irs * at4 - at5;
            pdot[3 * NC + ind] += coef * dd;
          }
        }
      }
      // derivatives of the force constants wrt rch(j) (opbend_ch4oh)
#pragma unroll
      for (int jb = 0; jb < 4; ++jb) {
        F ddr = F(fch3) * dsw[i][jb] * sum2 + F(hch3) * dsw[i][jb] * sum4;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          pdot[3 * NH(jb) + d] -= G.uch[jb][d] * ddr;
          pdot[3 * NC + d] += G.uch[jb][d] * ddr;
        }
      }
    }
  }

  // ---- in-plane bends (ipbend_ch4oh, ipforce_ch4oh)
  F vip = F(0);
  {
    const F f0 = F(fkinf + ak), g0 = F((fkinf + ak) - fkinf);  // f0 - f2
    F f1[4], df1dc[4], df1dh[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const F rb = G.rbh[i], xh = rb - F(r0hh), x = G.rch[i] - F(r0ch);
      F ea1 = t_exp<F>(-F(aa1) * rb * rb), ea2 = t_exp<F>(-F(aa4) * xh * xh);
      F a1 = F(1) - ea1, a2 = F(aa2) + F(aa3) * ea2;
      F eg = t_exp<F>(-a2 * (x * x));
      f1[i] = a1 * eg;
      F duma1 = F(2.0 * aa1) * rb * ea1;
      F duma2 = F(-2.0 * aa3 * aa4) * xh * ea2;
      df1dc[i] = F(-2) * x * a1 * a2 * eg;
      df1dh[i] = duma1 * eg - duma2 * (x * x) * a1 * eg;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = i + 1; j < 4; ++j) {
        int m = -1, n = -1;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (k != i && k != j) {
            if (m < 0) m = k;
            else n = k;
          }
        const F fk0 = f0 + f0 * (s1[i] * s1[j] - F(1)) + g0 * (s2[m] * s2[n] - F(1));
        F dfk0[4];
        dfk0[i] = f0 * ds1[i] * s1[j];
        dfk0[j] = f0 * s1[i] * ds1[j];
        dfk0[m] = g0 * ds2[m] * s2[n];
        dfk0[n] = g0 * s2[m] * ds2[n];
        const F kf = fk0 * f1[i] * f1[j];
        F costh, dth;
        if constexpr (kPair) {
          // theta - tau as asin(sin(theta - tau)) from a float-pair cosine:
          // theta - th0 is a small difference of two ~1.9 rad angles
          const ff c = (Xtch[i][0] * Xtch[j][0] + Xtch[i][1] * Xtch[j][1] + Xtch[i][2] * Xtch[j][2]) /
                       (Xrch[i] * Xrch[j]);
          constexpr ff kCosTau = ff_const(-1.0 / 3.0), kSinTau = ff_const(0.94280904158206336587);
          const ff y = ff_sqrt(ff_from(1.f) - c * c) * kCosTau - c * kSinTau;
          costh = ff_float(c);
          const float dtau = fabsf(y.hi) < 0.9f ? asinf(y.hi) + y.lo / sqrtf(1.f - y.hi * y.hi)
                                                : acosf(costh) - F(tau);
          dth = dtau - th0m[i][j];
        } else {
          costh = (G.uch[i][0] * G.uch[j][0] + G.uch[i][1] * G.uch[j][1] + G.uch[i][2] * G.uch[j][2]);
          dth = t_acos<F>(costh) - th0[i][j];
        }
        vip += F(0.5) * kf * dth * dth;
        const F termth = F(-1) / t_sqrt<F>(F(1) - costh * costh);
        const F half_d2 = F(0.5) * dth * dth;
#pragma unroll
        for (int ind = 0; ind < 3; ++ind) {
          F dthi = (-G.uch[j][ind] + costh * G.uch[i][ind]) * G.irch[i] * termth;
          F dthj = (-G.uch[i][ind] + costh * G.uch[j][ind]) * G.irch[j] * termth;
          pdot[3 * NH(i) + ind] += kf * dthi * dth;
          pdot[3 * NH(j) + ind] += kf * dthj * dth;
          pdot[3 * NC + ind] -= kf * (dthi + dthj) * dth;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            F dfdc = dfk0[k] * f1[i] * f1[j];
            if (k == i) dfdc += fk0 * df1dc[i] * f1[j];
            if (k == j) dfdc += fk0 * f1[i] * df1dc[j];
            F dfdh = F(0);
            if (k == i) dfdh = fk0 * df1dh[i] * f1[j];
            if (k == j) dfdh = fk0 * f1[i] * df1dh[j];
            const F dth0k = -dth0[i][j][k] * G.uch[k][ind];
            const F tc = G.uch[k][ind] * dfdc * half_d2;
            const F tb = G.tbh[k][ind] * G.irbh[k] * dfdh * half_d2;
            pdot[3 * NH(k) + ind] += -tc - tb - kf * dth0k * dth;
            pdot[3 * NC + ind] += tc + kf * dth0k * dth;
            pdot[3 * NB + ind] += tb;
          }
        }
      }
  }

  // ---- H(i)-O-H(O) bends (ipbend_ch4oh :1061-1172)
  {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const F* tb = G.tbh[i];
      F cosine, dang;
      if constexpr (kPair) {
        // angle - anh2oeq as asin(sin(angle - anh2oeq)) from a float-pair
        // cosine: a small difference of two ~1.8 rad angles
        const ff rno = ff_sqrt(Xtno[0] * Xtno[0] + Xtno[1] * Xtno[1] + Xtno[2] * Xtno[2]);
        const ff rbh = ff_sqrt(Xtbh[i][0] * Xtbh[i][0] + Xtbh[i][1] * Xtbh[i][1] + Xtbh[i][2] * Xtbh[i][2]);
        ff c = -((Xtno[0] * Xtbh[i][0] + Xtno[1] * Xtbh[i][1] + Xtno[2] * Xtbh[i][2]) / (rno * rbh));
        if (c.hi > 1.f) c = ff_from(1.f);
        if (c.hi < -1.f) c = ff_from(-1.f);
        constexpr ff kCosEq = ff_const(-0.25398078034139054), kSinEq = ff_const(0.9672092654731852);
        const ff y = ff_sqrt(ff_from(1.f) - c * c) * kCosEq - c * kSinEq;  // sin(angle - anh2oeq)
        cosine = ff_float(c);
        dang = fabsf(y.hi) < 0.9f ? asinf(y.hi) + y.lo / sqrtf(1.f - y.hi * y.hi)
                                  : t_acos<F>(cosine) - F(anh2oeq);
      } else {
        cosine = -(G.tno[0] * tb[0] + G.tno[1] * tb[1] + G.tno[2] * tb[2]) * (G.irno * G.irbh[i]);
        cosine = fmin(F(1), fmax(F(-1), cosine));
        dang = t_acos<F>(cosine) - F(anh2oeq);
      }
      const F arga = F(alph2o) * (G.rbh[i] - F(r0hh));
      const F fk = (arga < F(19.0)) ? F(fkh2oeq) * (F(1) - t_tanh<F>(arga)) : F(0);
      vip += F(0.5) * fk * dang * dang;
      const F deno = t_cosh<F>(arga);
      const F dkdr = -F(fkh2oeq * alph2o) / (deno * deno) * G.irbh[i];
      const F term1 = F(0.5) * dang * dang;
      const F dstda = fk * dang;
      const F xp = G.tno[1] * tb[2] - G.tno[2] * tb[1];
      const F yp = G.tno[2] * tb[0] - G.tno[0] * tb[2];
      const F zp = G.tno[0] * tb[1] - G.tno[1] * tb[0];
      F rp = t_sqrt<F>(xp * xp + yp * yp + zp * zp);
      if (rp < F(1.0e-6)) rp = F(1.0e-6);
      const F terma = dstda / (G.rbh[i] * G.rbh[i] * rp);
      const F termc = dstda / (G.rno * G.rno * rp);
      const F dedhi[3] = {-terma * (tb[1] * zp - tb[2] * yp), -terma * (tb[2] * xp - tb[0] * zp),
                          -terma * (tb[0] * yp - tb[1] * xp)};
      const F dedho[3] = {-termc * (G.tno[1] * zp - G.tno[2] * yp), -termc * (G.tno[2] * xp - G.tno[0] * zp),
                          -termc * (G.tno[0] * yp - G.tno[1] * xp)};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const F dk = dkdr * tb[d] * term1;
        pdot[3 * NB + d] += dk - dedhi[d] - dedho[d];
        pdot[3 * NH(i) + d] += -dk + dedhi[d];
        pdot[3 * NO + d] += dedho[d];
      }
    }
  }

  Vout = (double)((vstr + vop + vip) * F(0.03812));
  if constexpr (kPair) {
#pragma unroll
    for (int x = 0; x < 21; ++x) pdot[x] = ff_float(psx[x] + pdot[x]);
  }
#pragma unroll
  for (int x = 0; x < 21; ++x) gout[x] = (double)pdot[x] * 0.0201723;
}

}  // namespace ch4oh

struct PesCH4OH {
  static constexpr int N = 7;
  template <class F>
  __device__ static inline void egrad(const double (&q)[21], double& V, double (&g)[21]) {
    ch4oh::egrad<F, ch4oh::ParCH4OH>(q, V, g);
  }
};

// GeH4 + OH (src/egrad_geh4oh.f, Espinosa-Garcia, Rangel, Corchado, Phys.
// Chem. Chem. Phys. 18, 16941 (2016)): the CH4 + OH functional forms and atom
// roles (Ge in C's place) with its own constants.
struct PesGeH4OH {
  static constexpr int N = 7;
  template <class F>
  __device__ static inline void egrad(const double (&q)[21], double& V, double (&g)[21]) {
    ch4oh::egrad<F, ch4oh::ParGeH4OH>(q, V, g);
  }
};

}  // namespace cr
