// ORACLE (test infrastructure only) -- CH4 + OH potential, CPU restatement.
//
// Restates Caracal's src/egrad_ch4oh.f (the POTLIB surface of Espinosa-Garcia
// and Corchado, J. Chem. Phys. 112, 5731 (2000)) for one bead, with
// Caracal's settings of the POTLIB wrapper (src/util_ch4oh.f, identical to
// the CH4 + H one): bohr and Hartree user units, no atom relabelling,
// Cartesian R, ANUZERO = 0, so the wrapper routines are identities.
// Routine map (src/egrad_ch4oh.f):
//   egrad_ch4oh :69-124    q(3,7) -> V, dVdq
//   POT_ch4oh   :157-286   bohr -> Angstrom (x0.52918), energy x0.03812,
//               gradient x0.0201723
//   coorden :288  refangles :374  opbend :782  calcdelta :1177
//   opforce :1435  ipforce :1549  switchf :1748 (original POTLIB a1s..b2s):
//               as for CH4 + H
//   stretch :517  adds the switched C-B triplet depth d3cb(rav) (inert for
//               a3cb = 0 but evaluated) and the O-H Morse term
//   ipbend  :938  adds the four H(i)-O-H(O) harmonic bends with the
//               tanh-switched force constant fkh2o(rbh(i))
//   PREPOT  :1888 unit conversions (fact1, fact2, fact3 = 2 pi/360 for anh2oeq)
// Atom roles (BLOCK DATA): nnc = 2 (C), nnb = 6 (O), nnh = (3,4,5,1),
// nno = 7 (the hydroxyl H).  All constants are REAL(8).
// GeH4 + OH (src/egrad_geh4oh.f, Espinosa-Garcia, Rangel, Corchado, Phys.
// Chem. Chem. Phys. 18, 16941 (2016)) is the same code with its own BLOCK
// DATA (Ge in C's place), refangles' pyramid angle taugeh = 0.678 pi in place
// of halfpi (:368-392) and switchf's sphi without the rch < 3.8 condition
// (:1792-1804): params(true).
// Loop and accumulation orders follow the Fortran.
#pragma once
#include <cmath>

namespace orc {
namespace ch4oh {

using std::acos;
using std::cosh;
using std::exp;
using std::fmax;
using std::fmin;
using std::pow;
using std::sqrt;
using std::tanh;

struct Params {
  double r0ch, d1ch, d3ch, a1ch, b1ch, c1ch, r0hh, d1hh, d3hh, ahh, r0cb, d1cb, d3cbi, acb;
  double a3s, b3s, aphi, bphi, cphi, atheta, btheta, ctheta, fch3, hch3, fkinf, ak, bk;
  double aa1, aa2, aa3, aa4, fkh2oeq, alph2o, anh2oeq, a3cb, b3cb, rcbsp;
  double tau_py;   // refangles' pyramid angle: halfpi (CH4 + OH), taugeh = 0.678 pi (GeH4 + OH)
  bool sphi_cut;   // switchf's rch < 3.8 condition on sphi (absent in GeH4 + OH)
};

// PREPOT_ch4oh's unit conversions (src/egrad_ch4oh.f:1987-2003).
inline Params convert(Params q) {
  const double pi = 3.141592653589793;
  const double fact1 = 0.041840, fact2 = 6.022045, fact3 = 2.0 * pi / 360.0;
  q.d1ch *= fact1; q.d3ch *= fact1; q.d1cb *= fact1; q.d3cbi *= fact1; q.a3cb *= fact1;
  q.d1hh *= fact1; q.d3hh *= fact1;
  q.fch3 *= fact2; q.hch3 *= fact2; q.fkinf *= fact2; q.ak *= fact2; q.fkh2oeq *= fact2;
  q.anh2oeq *= fact3;
  return q;
}

// BLOCK DATA PTPACM_ch4oh values after PREPOT_ch4oh's conversions, or with
// geh4oh those of PTPACM_geh4oh (src/egrad_geh4oh.f:2001-2045) after
// initialize_geh4oh's (the same conversions).
inline const Params& params(bool geh4oh = false) {
  static const Params p_ch4oh = [] {
    Params q;
    q.r0ch = 1.09397;  q.d1ch = 112.17000; q.d3ch = 32.65328;  q.a1ch = 1.78000;
    q.b1ch = 0.15000;  q.c1ch = 15.00000;  q.r0hh = 0.97060;   q.d1hh = 125.44000;
    q.d3hh = 20.41017; q.ahh = 2.15000;    q.r0cb = 1.49092;   q.d1cb = 91.47526;
    q.d3cbi = 112.69509; q.acb = 2.98688;  q.a3s = 0.1419100;  q.b3s = -0.3068400;
    q.aphi = 0.5287900; q.bphi = 0.4006600; q.cphi = 1.9209900; q.atheta = 0.9078700;
    q.btheta = 0.3548900; q.ctheta = 1.8915500; q.fch3 = 0.0740000; q.hch3 = 0.1915000;
    q.fkinf = 0.4400000; q.ak = 0.1260000; q.bk = 10.7132; q.aa1 = 0.303746;
    q.aa2 = 1.599960; q.aa3 = 3.216595; q.aa4 = 11.569980; q.fkh2oeq = 0.7300000;
    q.alph2o = 1.1080000; q.anh2oeq = 104.7132000; q.a3cb = 0.000000; q.b3cb = 0.900000;
    q.rcbsp = 2.606485;
    q.tau_py = 0.5 * 3.141592653589793;
    q.sphi_cut = true;
    return convert(q);
  }();
  static const Params p_geh4oh = [] {
    Params q;
    q.r0ch = 1.52500;  q.d1ch = 86.50000;  q.d3ch = 41.50000;  q.a1ch = 1.43925;
    q.b1ch = 0.12330;  q.c1ch = 2.00400;   q.r0hh = 0.97060;   q.d1hh = 120.94800;
    q.d3hh = 31.86417; q.ahh = 2.18200;    q.r0cb = 1.90035;   q.d1cb = 41.50283;
    q.d3cbi = 10.50589; q.acb = 0.67621;   q.a3s = 0.2019100;  q.b3s = -0.6068400;
    q.aphi = 0.5287900; q.bphi = 0.4006600; q.cphi = 11.8809900; q.atheta = 0.9078700;
    q.btheta = 0.3548900; q.ctheta = 1.8915500; q.fch3 = 0.0150000; q.hch3 = 0.1915000;
    q.fkinf = 0.3060000; q.ak = 0.1260000; q.bk = 50.7132; q.aa1 = 0.173746;
    q.aa2 = 1.599960; q.aa3 = 2.166595; q.aa4 = 11.569980; q.fkh2oeq = 0.7300000;
    q.alph2o = 1.1080000; q.anh2oeq = 104.7132000; q.a3cb = 0.000000; q.b3cb = 0.900000;
    q.rcbsp = 2.606485;
    q.tau_py = 0.678 * 3.141592653589793;
    q.sphi_cut = false;
    return convert(q);
  }();
  return geh4oh ? p_geh4oh : p_ch4oh;
}

// Working state of one evaluation (Caracal keeps it in COMMON blocks).
template <class T>
struct State {
  const Params* P;        // the surface's constants
  T q[22];                // q(1..21), Angstrom (1-based)
  T pdot[22];             // dE/dq(1..21)
  int nc[4], nhb[4], nh[5][4], no[4];  // coordinate indices, 1-based
  T tcb[4], tno[4], tch[5][4], tbh[5][4];
  T rcb, rno, rch[5], rbh[5];
  T s1[5], ds1[5], s2[5], ds2[5], s3[5], ds3[5], sphi[5], dsphi[5], stheta[5], dstheta[5];
  T theta0[5][5], dtheta0[5][5][5];
  T fdelta[5], hdelta[5], dfdelta[5][5], dhdelta[5][5];
  T fk0[5][5], f1[5], dfdc[5][5][5], dfdh[5][5][5];
};

template <class T>
inline T sq(T x) { return x * x; }

template <class T>
inline void coorden(State<T>& s) {
  for (int ind = 1; ind <= 3; ++ind) {
    s.tcb[ind] = s.q[s.nc[ind]] - s.q[s.nhb[ind]];
    s.tno[ind] = s.q[s.no[ind]] - s.q[s.nhb[ind]];
    for (int i = 1; i <= 4; ++i) {
      s.tch[i][ind] = s.q[s.nc[ind]] - s.q[s.nh[i][ind]];
      s.tbh[i][ind] = s.q[s.nhb[ind]] - s.q[s.nh[i][ind]];
    }
  }
  s.rcb = sqrt(s.tcb[1] * s.tcb[1] + s.tcb[2] * s.tcb[2] + s.tcb[3] * s.tcb[3]);
  s.rno = sqrt(s.tno[1] * s.tno[1] + s.tno[2] * s.tno[2] + s.tno[3] * s.tno[3]);
  for (int i = 1; i <= 4; ++i) {
    s.rch[i] = sqrt(s.tch[i][1] * s.tch[i][1] + s.tch[i][2] * s.tch[i][2] + s.tch[i][3] * s.tch[i][3]);
    s.rbh[i] = sqrt(s.tbh[i][1] * s.tbh[i][1] + s.tbh[i][2] * s.tbh[i][2] + s.tbh[i][3] * s.tbh[i][3]);
  }
}

template <class T>
inline void switchf(State<T>& s) {
  const Params& P = *s.P;
  const double a1s = 1.5313681e-7, b1s = -4.6696246, a2s = 1.0147402e-7, b2s = -12.363798;
  const double argmax = 19.0;
  for (int i = 1; i <= 4; ++i) {
    T r = s.rch[i];
    T x1 = r - b1s, x1_2 = x1 * x1, x1_4 = x1_2 * x1_2, x1_8 = x1_4 * x1_4, x1_7 = x1_4 * x1_2 * x1;
    T args1 = a1s * (r - P.r0ch) * x1_8;
    if (args1 < argmax) {
      s.s1[i] = 1.0 - tanh(args1);
      T d = a1s * (x1_8 + 8.0 * (r - P.r0ch) * x1_7);
      T ch = cosh(args1);
      s.ds1[i] = -d / (ch * ch);
    } else {
      s.s1[i] = 0.0;
      s.ds1[i] = 0.0;
    }
    T x2 = r - b2s, x2_2 = x2 * x2, x2_4 = x2_2 * x2_2, x2_6 = x2_4 * x2_2, x2_5 = x2_4 * x2;
    T args2 = a2s * (r - P.r0ch) * x2_6;
    if (args2 < argmax) {
      s.s2[i] = 1.0 - tanh(args2);
      T d = a2s * (x2_6 + 6.0 * (r - P.r0ch) * x2_5);
      T ch = cosh(args2);
      s.ds2[i] = -d / (ch * ch);
    } else {
      s.s2[i] = 0.0;
      s.ds2[i] = 0.0;
    }
    T args3 = P.a3s * (r - P.r0ch) * sq(r - P.b3s);
    if (args3 < argmax) {
      s.s3[i] = 1.0 - tanh(args3);
      T d = P.a3s * (3.0 * r * r - 2.0 * r * (P.r0ch + 2.0 * P.b3s) + P.b3s * (P.b3s + 2.0 * P.r0ch));
      T ch = cosh(args3);
      s.ds3[i] = -d / (ch * ch);
    } else {
      s.s3[i] = 0.0;
      s.ds3[i] = 0.0;
    }
    if (!P.sphi_cut || r < 3.8) {
      T xc = r - P.cphi;
      T e = exp(P.bphi * xc * xc * xc);
      T arg = P.aphi * (r - P.r0ch) * e;
      s.sphi[i] = 1.0 - tanh(arg);
      T d = P.aphi * (1.0 + 3.0 * P.bphi * (r - P.r0ch) * xc * xc);
      d = d * e;
      T ch = cosh(arg);
      s.dsphi[i] = -d / (ch * ch);
    } else {
      s.sphi[i] = 0.0;
      s.dsphi[i] = 0.0;
    }
    if (r < 3.8) {
      T xc = r - P.ctheta;
      T e = exp(P.btheta * xc * xc * xc);
      T arg = P.atheta * (r - P.r0ch) * e;
      s.stheta[i] = 1.0 - tanh(arg);
      T d = P.atheta * (1.0 + 3.0 * P.btheta * (r - P.r0ch) * xc * xc);
      d = d * e;
      T ch = cosh(arg);
      s.dstheta[i] = -d / (ch * ch);
    } else {
      s.stheta[i] = 0.0;
      s.dstheta[i] = 0.0;
    }
  }
}

template <class T>
inline void refangles(State<T>& s) {
  const double pi = 3.141592653589793;
  const double tau = std::acos(-1.0 / 3.0);
  const double twopi = 2.0 * pi;
  const double A = tau - s.P->tau_py, B = tau - twopi / 3.0;
  for (int i = 1; i <= 4; ++i) {
    s.theta0[i][i] = 0.0;
    for (int k = 1; k <= 4; ++k) s.dtheta0[i][i][k] = 0.0;
  }
  T* sp = s.sphi;
  T* st = s.stheta;
  T* dsp = s.dsphi;
  T* dst = s.dstheta;
  s.theta0[1][2] = tau + A * (sp[1] * sp[2] - 1.0) + B * (st[3] * st[4] - 1.0);
  s.theta0[1][3] = tau + A * (sp[1] * sp[3] - 1.0) + B * (st[2] * st[4] - 1.0);
  s.theta0[1][4] = tau + A * (sp[1] * sp[4] - 1.0) + B * (st[2] * st[3] - 1.0);
  s.theta0[2][3] = tau + A * (sp[2] * sp[3] - 1.0) + B * (st[1] * st[4] - 1.0);
  s.theta0[2][4] = tau + A * (sp[2] * sp[4] - 1.0) + B * (st[1] * st[3] - 1.0);
  s.theta0[3][4] = tau + A * (sp[3] * sp[4] - 1.0) + B * (st[1] * st[2] - 1.0);
  // wrt rch(1)
  s.dtheta0[1][2][1] = A * dsp[1] * sp[2];
  s.dtheta0[1][3][1] = A * dsp[1] * sp[3];
  s.dtheta0[1][4][1] = A * dsp[1] * sp[4];
  s.dtheta0[2][3][1] = B * dst[1] * st[4];
  s.dtheta0[2][4][1] = B * dst[1] * st[3];
  s.dtheta0[3][4][1] = B * dst[1] * st[2];
  // wrt rch(2)
  s.dtheta0[1][2][2] = A * sp[1] * dsp[2];
  s.dtheta0[1][3][2] = B * dst[2] * st[4];
  s.dtheta0[1][4][2] = B * dst[2] * st[3];
  s.dtheta0[2][3][2] = A * dsp[2] * sp[3];
  s.dtheta0[2][4][2] = A * dsp[2] * sp[4];
  s.dtheta0[3][4][2] = B * st[1] * dst[2];
  // wrt rch(3)
  s.dtheta0[1][2][3] = B * dst[3] * st[4];
  s.dtheta0[1][3][3] = A * sp[1] * dsp[3];
  s.dtheta0[1][4][3] = B * st[2] * dst[3];
  s.dtheta0[2][3][3] = A * sp[2] * dsp[3];
  s.dtheta0[2][4][3] = B * st[1] * dst[3];
  s.dtheta0[3][4][3] = A * dsp[3] * sp[4];
  // wrt rch(4)
  s.dtheta0[1][2][4] = B * st[3] * dst[4];
  s.dtheta0[1][3][4] = B * st[2] * dst[4];
  s.dtheta0[1][4][4] = A * sp[1] * dsp[4];
  s.dtheta0[2][3][4] = B * st[1] * dst[4];
  s.dtheta0[2][4][4] = A * sp[2] * dsp[4];
  s.dtheta0[3][4][4] = A * sp[3] * dsp[4];
  for (int i = 1; i <= 3; ++i)
    for (int j = i + 1; j <= 4; ++j) {
      s.theta0[j][i] = s.theta0[i][j];
      for (int k = 1; k <= 4; ++k) s.dtheta0[j][i][k] = s.dtheta0[i][j][k];
    }
}

template <class T>
inline void stretch(State<T>& s, T* vstr_out) {
  const Params& P = *s.P;
  T vqch[5], vjch[5], vqbh[5], vjbh[5], vq[5], vj[5], achdc[4], achdh[5][4];
  T rav = (s.rch[1] + s.rch[2] + s.rch[3] + s.rch[4]) / 4.0;
  T vstr = 0.0;
  // switched triplet depth of C-B (src/egrad_ch4oh.f:581-583)
  T texp = exp(-pow(4.0 * (rav - P.rcbsp) / P.b3cb, T(4.0)));
  T d3cb = (P.d3cbi - P.a3cb) + P.a3cb * texp;
  T dd3cb = -4.0 * P.a3cb * texp * pow(rav - P.rcbsp, T(3.0)) * pow(T(4.0 / P.b3cb), T(4.0));
  T arga = P.c1ch * (rav - P.r0ch);
  T ach, dumach;
  if (arga < 19.0) {
    ach = P.a1ch + P.b1ch * (tanh(arga) + 1.0) * 0.5;
    T ch = cosh(arga);
    dumach = P.b1ch * P.c1ch / (2.0 * (ch * ch));
  } else {
    ach = P.a1ch + P.b1ch;
    dumach = 0.0;
  }
  T ecb2 = exp(-2.0 * P.acb * (s.rcb - P.r0cb)), ecb1 = exp(-P.acb * (s.rcb - P.r0cb));
  T e1 = P.d1cb * (ecb2 - 2.0 * ecb1);
  T e3 = d3cb * (ecb2 + 2.0 * ecb1);
  T vqcb = (e1 + e3) * 0.5;
  T vjcb = (e1 - e3) * 0.5;
  // O-H Morse term
  T dt = s.rno - P.r0hh;
  T expterm = exp(-P.ahh * dt);
  T vno = P.d1hh * sq(1.0 - expterm);
  for (int i = 1; i <= 4; ++i) {
    T ec2 = exp(-2.0 * ach * (s.rch[i] - P.r0ch)), ec1 = exp(-ach * (s.rch[i] - P.r0ch));
    e1 = P.d1ch * (ec2 - 2.0 * ec1);
    e3 = P.d3ch * (ec2 + 2.0 * ec1);
    vqch[i] = (e1 + e3) * 0.5;
    vjch[i] = (e1 - e3) * 0.5;
    T eh2 = exp(-2.0 * P.ahh * (s.rbh[i] - P.r0hh)), eh1 = exp(-P.ahh * (s.rbh[i] - P.r0hh));
    e1 = P.d1hh * (eh2 - 2.0 * eh1);
    e3 = P.d3hh * (eh2 + 2.0 * eh1);
    vqbh[i] = (e1 + e3) * 0.5;
    vjbh[i] = (e1 - e3) * 0.5;
    vq[i] = vqch[i] + vqcb + vqbh[i];
    vj[i] = -sqrt((sq(vjch[i] - vjcb) + sq(vjcb - vjbh[i]) + sq(vjbh[i] - vjch[i])) * 0.5);
    vstr = vstr + vq[i] + vj[i];
  }
  vstr = vstr + vno;
  T deddt = 2.0 * P.ahh * P.d1hh * (1.0 - expterm) * expterm;
  T de = deddt / s.rno;
  T ded[4];
  for (int i = 1; i <= 3; ++i) ded[i] = de * s.tno[i];
  for (int ind = 1; ind <= 3; ++ind) {
    achdc[ind] = dumach *
                 (s.tch[1][ind] / s.rch[1] + s.tch[2][ind] / s.rch[2] + s.tch[3][ind] / s.rch[3] +
                  s.tch[4][ind] / s.rch[4]) / 4.0;
    for (int i = 1; i <= 4; ++i) achdh[i][ind] = -dumach * s.tch[i][ind] / s.rch[i] / 4.0;
  }
  T dumqcb = -P.acb * ((P.d1cb + d3cb) * ecb2 - (P.d1cb - d3cb) * ecb1) / s.rcb;
  for (int i = 1; i <= 4; ++i) {
    T eh2 = exp(-2.0 * P.ahh * (s.rbh[i] - P.r0hh)), eh1 = exp(-P.ahh * (s.rbh[i] - P.r0hh));
    T ec2 = exp(-2.0 * ach * (s.rch[i] - P.r0ch)), ec1 = exp(-ach * (s.rch[i] - P.r0ch));
    T dumqbh = -P.ahh * ((P.d1hh + P.d3hh) * eh2 - (P.d1hh - P.d3hh) * eh1) / s.rbh[i];
    T addd3 = dd3cb * (exp(-2.0 * P.acb * (s.rcb - P.r0cb)) + 2.0 * exp(-P.acb * (s.rcb - P.r0cb)));
    addd3 = addd3 / 4.0 * 0.5 / s.rcb;
    dumqbh = dumqbh + addd3;
    T factj = 0.5 / vj[i];
    T dumjcb = -P.acb * ((P.d1cb - d3cb) * ecb2 - (P.d1cb + d3cb) * ecb1) * factj / s.rcb;
    T dumjbh = -P.ahh * ((P.d1hh - P.d3hh) * eh2 - (P.d1hh + P.d3hh) * eh1) * factj / s.rbh[i];
    addd3 = dd3cb * (exp(-2.0 * P.acb * (s.rcb - P.r0cb)) + 2.0 * exp(-P.acb * (s.rcb - P.r0cb)));
    addd3 = addd3 / 4.0 * 0.5 * factj / s.rcb;
    dumjbh = dumjbh - addd3;
    for (int ind = 1; ind <= 3; ++ind) {
      T& pb = s.pdot[s.nhb[ind]];
      pb = pb - s.tcb[ind] * dumqcb + s.tbh[i][ind] * dumqbh + (vjch[i] - vjcb) * (dumjcb * s.tcb[ind]) +
           (vjcb - vjbh[i]) * (-dumjcb * s.tcb[ind] - dumjbh * s.tbh[i][ind]) +
           (vjbh[i] - vjch[i]) * dumjbh * s.tbh[i][ind];
      T brq = (P.d1ch + P.d3ch) * ec2 - (P.d1ch - P.d3ch) * ec1;
      T brj = (P.d1ch - P.d3ch) * ec2 - (P.d1ch + P.d3ch) * ec1;
      T dumqch = -(ach * s.tch[i][ind] / s.rch[i] + achdc[ind] * (s.rch[i] - P.r0ch)) * brq;
      T& pc = s.pdot[s.nc[ind]];
      pc = pc + dumqch + s.tcb[ind] * dumqcb;
      T dumqhi = (ach * s.tch[i][ind] / s.rch[i] - achdh[i][ind] * (s.rch[i] - P.r0ch)) * brq;
      T& ph = s.pdot[s.nh[i][ind]];
      ph = ph + dumqhi - s.tbh[i][ind] * dumqbh;
      T dumjch = -(ach * s.tch[i][ind] / s.rch[i] + achdc[ind] * (s.rch[i] - P.r0ch)) * brj * factj;
      pc = pc + (vjch[i] - vjcb) * (dumjch - dumjcb * s.tcb[ind]) + (vjcb - vjbh[i]) * dumjcb * s.tcb[ind] -
           (vjbh[i] - vjch[i]) * dumjch;
      T dumjhi = (ach * s.tch[i][ind] / s.rch[i] - achdh[i][ind] * (s.rch[i] - P.r0ch)) * brj * factj;
      ph = ph + (vjch[i] - vjcb) * dumjhi + (vjcb - vjbh[i]) * dumjbh * s.tbh[i][ind] +
           (vjbh[i] - vjch[i]) * (-dumjbh * s.tbh[i][ind] - dumjhi);
      for (int k = 1; k <= 3; ++k) {
        int j = i + k;
        if (j > 4) j = j - 4;
        T dumqhj = -achdh[j][ind] * (s.rch[i] - P.r0ch) * brq;
        T dumjhj = -achdh[j][ind] * (s.rch[i] - P.r0ch) * brj * factj;
        T& pj = s.pdot[s.nh[j][ind]];
        pj = pj + dumqhj + (vjch[i] - vjcb) * dumjhj - (vjbh[i] - vjch[i]) * dumjhj;
      }
    }
  }
  for (int ind = 1; ind <= 3; ++ind) {
    s.pdot[s.nhb[ind]] = s.pdot[s.nhb[ind]] - ded[ind];
    s.pdot[s.no[ind]] = s.pdot[s.no[ind]] + ded[ind];
  }
  *vstr_out = vstr;
}

template <class T>
inline void opforce(State<T>& s) {
  const Params& P = *s.P;
  T* s3 = s.s3;
  T* ds3 = s.ds3;
  T sw[5], dsw[5][5];
  sw[1] = (1.0 - s3[1]) * s3[2] * s3[3] * s3[4];
  sw[2] = (1.0 - s3[2]) * s3[3] * s3[4] * s3[1];
  sw[3] = (1.0 - s3[3]) * s3[4] * s3[1] * s3[2];
  sw[4] = (1.0 - s3[4]) * s3[1] * s3[2] * s3[3];
  dsw[1][1] = -ds3[1] * s3[2] * s3[3] * s3[4];
  dsw[1][2] = (1.0 - s3[1]) * ds3[2] * s3[3] * s3[4];
  dsw[1][3] = (1.0 - s3[1]) * s3[2] * ds3[3] * s3[4];
  dsw[1][4] = (1.0 - s3[1]) * s3[2] * s3[3] * ds3[4];
  dsw[2][1] = (1.0 - s3[2]) * s3[3] * s3[4] * ds3[1];
  dsw[2][2] = -ds3[2] * s3[3] * s3[4] * s3[1];
  dsw[2][3] = (1.0 - s3[2]) * ds3[3] * s3[4] * s3[1];
  dsw[2][4] = (1.0 - s3[2]) * s3[3] * ds3[4] * s3[1];
  dsw[3][1] = (1.0 - s3[3]) * s3[4] * ds3[1] * s3[2];
  dsw[3][2] = (1.0 - s3[3]) * s3[4] * s3[1] * ds3[2];
  dsw[3][3] = -ds3[3] * s3[4] * s3[1] * s3[2];
  dsw[3][4] = (1.0 - s3[3]) * ds3[4] * s3[1] * s3[2];
  dsw[4][1] = (1.0 - s3[4]) * ds3[1] * s3[2] * s3[3];
  dsw[4][2] = (1.0 - s3[4]) * s3[1] * ds3[2] * s3[3];
  dsw[4][3] = (1.0 - s3[4]) * s3[1] * s3[2] * ds3[3];
  dsw[4][4] = -ds3[4] * s3[1] * s3[2] * s3[3];
  for (int i = 1; i <= 4; ++i) {
    s.fdelta[i] = sw[i] * P.fch3;
    s.hdelta[i] = sw[i] * P.hch3;
    for (int j = 1; j <= 4; ++j) {
      s.dfdelta[i][j] = dsw[i][j] * P.fch3;
      s.dhdelta[i][j] = dsw[i][j] * P.hch3;
    }
  }
}

template <class T>
inline void calcdelta(State<T>& s, int i, int j, int k, int l, T* sum2, T* sum4) {
  T delta[5], a[4], b[4], axb[4], c[5][4], argd[5], daxb[5][4][4], cdot[5][4][4], atemp2[4];
  int in[4] = {0, j, k, l};
  T s2 = 0.0, s4 = 0.0;
  for (int ind = 1; ind <= 3; ++ind) {
    a[ind] = s.q[s.nh[k][ind]] - s.q[s.nh[j][ind]];
    b[ind] = s.q[s.nh[l][ind]] - s.q[s.nh[j][ind]];
  }
  axb[1] = a[2] * b[3] - a[3] * b[2];
  axb[2] = a[3] * b[1] - a[1] * b[3];
  axb[3] = a[1] * b[2] - a[2] * b[1];
  T norma = axb[1] * axb[1] + axb[2] * axb[2] + axb[3] * axb[3];
  norma = sqrt(norma);
  for (int ii = 1; ii <= 3; ++ii)
    for (int ind = 1; ind <= 3; ++ind) c[in[ii]][ind] = -s.tch[in[ii]][ind] / s.rch[in[ii]];
  for (int ii = 1; ii <= 3; ++ii) {
    argd[in[ii]] = axb[1] * c[in[ii]][1] + axb[2] * c[in[ii]][2] + axb[3] * c[in[ii]][3];
    argd[in[ii]] = argd[in[ii]] / norma;
    delta[in[ii]] = acos(argd[in[ii]]) - s.theta0[i][in[ii]];
    T d2 = delta[in[ii]] * delta[in[ii]];
    s2 = s2 + d2;
    s4 = s4 + d2 * d2;
  }
  // derivatives of axb wrt h_j, h_k, h_l
  daxb[j][1][1] = 0.0;         daxb[j][1][2] = b[3] - a[3];  daxb[j][1][3] = -b[2] + a[2];
  daxb[j][2][1] = -b[3] + a[3]; daxb[j][2][2] = 0.0;         daxb[j][2][3] = b[1] - a[1];
  daxb[j][3][1] = b[2] - a[2];  daxb[j][3][2] = -b[1] + a[1]; daxb[j][3][3] = 0.0;
  daxb[k][1][1] = 0.0;   daxb[k][1][2] = -b[3]; daxb[k][1][3] = b[2];
  daxb[k][2][1] = b[3];  daxb[k][2][2] = 0.0;   daxb[k][2][3] = -b[1];
  daxb[k][3][1] = -b[2]; daxb[k][3][2] = b[1];  daxb[k][3][3] = 0.0;
  daxb[l][1][1] = 0.0;   daxb[l][1][2] = a[3];  daxb[l][1][3] = -a[2];
  daxb[l][2][1] = -a[3]; daxb[l][2][2] = 0.0;   daxb[l][2][3] = a[1];
  daxb[l][3][1] = a[2];  daxb[l][3][2] = -a[1]; daxb[l][3][3] = 0.0;
  for (int ii = 1; ii <= 3; ++ii) {
    const int m = in[ii];
    T r2 = s.rch[m] * s.rch[m];
    cdot[m][1][1] = 1.0 / s.rch[m] + s.tch[m][1] * c[m][1] / r2;
    cdot[m][1][2] = s.tch[m][2] * c[m][1] / r2;
    cdot[m][1][3] = s.tch[m][3] * c[m][1] / r2;
    cdot[m][2][1] = s.tch[m][1] * c[m][2] / r2;
    cdot[m][2][2] = 1.0 / s.rch[m] + s.tch[m][2] * c[m][2] / r2;
    cdot[m][2][3] = s.tch[m][3] * c[m][2] / r2;
    cdot[m][3][1] = s.tch[m][1] * c[m][3] / r2;
    cdot[m][3][2] = s.tch[m][2] * c[m][3] / r2;
    cdot[m][3][3] = 1.0 / s.rch[m] + s.tch[m][3] * c[m][3] / r2;
  }
  for (int ii = 1; ii <= 3; ++ii) {
    for (int ind = 1; ind <= 3; ++ind) {
      const int m = in[ii];
      T dm = delta[m], dm3 = dm * dm * dm;
      T deldot = -s.dtheta0[i][m][i];
      deldot = -deldot * s.tch[i][ind] / s.rch[i];
      T& phi = s.pdot[s.nh[i][ind]];
      phi = phi + 2.0 * s.fdelta[i] * dm * deldot + 4.0 * s.hdelta[i] * dm3 * deldot;
      deldot = -deldot;
      T& pc = s.pdot[s.nc[ind]];
      pc = pc + 2.0 * s.fdelta[i] * dm * deldot + 4.0 * s.hdelta[i] * dm3 * deldot;
      for (int jj = 1; jj <= 3; ++jj) {
        const int mj = in[jj];
        T atemp1 = axb[1] * daxb[mj][ind][1] + axb[2] * daxb[mj][ind][2] + axb[3] * daxb[mj][ind][3];
        atemp1 = atemp1 / (norma * norma * norma);
        atemp2[1] = daxb[mj][ind][1] / norma - atemp1 * axb[1];
        atemp2[2] = daxb[mj][ind][2] / norma - atemp1 * axb[2];
        atemp2[3] = daxb[mj][ind][3] / norma - atemp1 * axb[3];
        T atemp3 = atemp2[1] * c[m][1] + atemp2[2] * c[m][2] + atemp2[3] * c[m][3];
        T atemp4 = 0.0;
        if (ii == jj) {
          atemp4 = axb[1] * cdot[m][1][ind] + axb[2] * cdot[m][2][ind] + axb[3] * cdot[m][3][ind];
          atemp4 = atemp4 / norma;
        }
        T atemp5 = -s.dtheta0[i][m][mj];
        atemp5 = -atemp5 * s.tch[mj][ind] / s.rch[mj];
        deldot = atemp3 + atemp4;
        T rs = sqrt(1.0 - argd[m] * argd[m]);
        deldot = -1.0 / rs * deldot;
        deldot = deldot + atemp5;
        T& pj = s.pdot[s.nh[mj][ind]];
        pj = pj + 2.0 * s.fdelta[i] * dm * deldot + 4.0 * s.hdelta[i] * dm3 * deldot;
        deldot = 1.0 / rs * atemp4;
        deldot = deldot - atemp5;
        pc = pc + 2.0 * s.fdelta[i] * dm * deldot + 4.0 * s.hdelta[i] * dm3 * deldot;
      }
    }
  }
  *sum2 = s2;
  *sum4 = s4;
}

template <class T>
inline void opbend(State<T>& s, T* vop_out) {
  T vop = 0.0, sumd2[5], sumd4[5];
  opforce(s);
  for (int i = 1; i <= 4; ++i) {
    int j = i + 1;
    if (j > 4) j = j - 4;
    int k = j + 1;
    if (k > 4) k = k - 4;
    int l = k + 1;
    if (l > 4) l = l - 4;
    int in[4] = {0, j, k, l};
    T a[4], b[4], axb[4], c[5][4];
    for (int ind = 1; ind <= 3; ++ind) {
      a[ind] = s.q[s.nh[k][ind]] - s.q[s.nh[j][ind]];
      b[ind] = s.q[s.nh[l][ind]] - s.q[s.nh[j][ind]];
    }
    axb[1] = a[2] * b[3] - a[3] * b[2];
    axb[2] = a[3] * b[1] - a[1] * b[3];
    axb[3] = a[1] * b[2] - a[2] * b[1];
    T norma = sqrt(axb[1] * axb[1] + axb[2] * axb[2] + axb[3] * axb[3]);
    for (int ii = 1; ii <= 3; ++ii)
      for (int ind = 1; ind <= 3; ++ind) c[in[ii]][ind] = -s.tch[in[ii]][ind] / s.rch[in[ii]];
    for (int ii = 1; ii <= 3; ++ii) {
      T argd = axb[1] * c[in[ii]][1] + axb[2] * c[in[ii]][2] + axb[3] * c[in[ii]][3];
      argd = argd / norma;
      if (argd > 0.0) {  // make (rj, rk, rl) right-handed: swap k and l
        int t = k;
        k = l;
        l = t;
      }
    }
    T sum2, sum4;
    calcdelta(s, i, j, k, l, &sum2, &sum4);
    sumd2[i] = sum2;
    sumd4[i] = sum4;
    vop = vop + s.fdelta[i] * sumd2[i] + s.hdelta[i] * sumd4[i];
  }
  for (int i = 1; i <= 4; ++i)
    for (int j = 1; j <= 4; ++j) {
      T ddr = s.dfdelta[i][j] * sumd2[i] + s.dhdelta[i][j] * sumd4[i];
      for (int ind = 1; ind <= 3; ++ind) {
        s.pdot[s.nh[j][ind]] = s.pdot[s.nh[j][ind]] - s.tch[j][ind] * ddr / s.rch[j];
        s.pdot[s.nc[ind]] = s.pdot[s.nc[ind]] + s.tch[j][ind] * ddr / s.rch[j];
      }
    }
  *vop_out = vop;
}

template <class T>
inline void ipforce(State<T>& s) {
  const Params& P = *s.P;
  T dfk0[5][5][5], df1dc[5], df1dh[5];
  T* s1 = s.s1;
  T* s2 = s.s2;
  T* ds1 = s.ds1;
  T* ds2 = s.ds2;
  const double f0 = P.fkinf + P.ak, f2 = P.fkinf;
  const double g = f0 - f2;
  s.fk0[1][2] = f0 + f0 * (s1[1] * s1[2] - 1.0) + g * (s2[3] * s2[4] - 1.0);
  s.fk0[1][3] = f0 + f0 * (s1[1] * s1[3] - 1.0) + g * (s2[2] * s2[4] - 1.0);
  s.fk0[1][4] = f0 + f0 * (s1[1] * s1[4] - 1.0) + g * (s2[2] * s2[3] - 1.0);
  s.fk0[2][3] = f0 + f0 * (s1[2] * s1[3] - 1.0) + g * (s2[1] * s2[4] - 1.0);
  s.fk0[2][4] = f0 + f0 * (s1[2] * s1[4] - 1.0) + g * (s2[1] * s2[3] - 1.0);
  s.fk0[3][4] = f0 + f0 * (s1[3] * s1[4] - 1.0) + g * (s2[1] * s2[2] - 1.0);
  dfk0[1][2][1] = f0 * ds1[1] * s1[2];
  dfk0[1][2][2] = f0 * s1[1] * ds1[2];
  dfk0[1][2][3] = g * ds2[3] * s2[4];
  dfk0[1][2][4] = g * s2[3] * ds2[4];
  dfk0[1][3][1] = f0 * ds1[1] * s1[3];
  dfk0[1][3][2] = g * ds2[2] * s2[4];
  dfk0[1][3][3] = f0 * s1[1] * ds1[3];
  dfk0[1][3][4] = g * s2[2] * ds2[4];
  dfk0[1][4][1] = f0 * ds1[1] * s1[4];
  dfk0[1][4][2] = g * ds2[2] * s2[3];
  dfk0[1][4][3] = g * s2[2] * ds2[3];
  dfk0[1][4][4] = f0 * s1[1] * ds1[4];
  dfk0[2][3][1] = g * ds2[1] * s2[4];
  dfk0[2][3][2] = f0 * ds1[2] * s1[3];
  dfk0[2][3][3] = f0 * s1[2] * ds1[3];
  dfk0[2][3][4] = g * s2[1] * ds2[4];
  dfk0[2][4][1] = g * ds2[1] * s2[3];
  dfk0[2][4][2] = f0 * ds1[2] * s1[4];
  dfk0[2][4][3] = g * s2[1] * ds2[3];
  dfk0[2][4][4] = f0 * s1[2] * ds1[4];
  dfk0[3][4][1] = g * ds2[1] * s2[2];
  dfk0[3][4][2] = g * s2[1] * ds2[2];
  dfk0[3][4][3] = f0 * ds1[3] * s1[4];
  dfk0[3][4][4] = f0 * s1[3] * ds1[4];
  for (int i = 1; i <= 4; ++i) {
    T arga1 = P.aa1 * s.rbh[i] * s.rbh[i];
    T arga2 = P.aa4 * (s.rbh[i] - P.r0hh) * (s.rbh[i] - P.r0hh);
    T ea1 = exp(-arga1), ea2 = exp(-arga2);
    T a1 = 1.0 - ea1;
    T a2 = P.aa2 + P.aa3 * ea2;
    T x = s.rch[i] - P.r0ch;
    T eg = exp(-a2 * (x * x));
    s.f1[i] = a1 * eg;
    T duma1 = 2.0 * P.aa1 * s.rbh[i] * ea1;
    T duma2 = -2.0 * P.aa3 * P.aa4 * (s.rbh[i] - P.r0hh) * ea2;
    df1dc[i] = -2.0 * x * a1 * a2 * eg;
    df1dh[i] = duma1 * eg - duma2 * (x * x) * a1 * eg;
  }
  T* f1 = s.f1;
  // dfdc(i,j,k): derivative of fk0(i,j) f1(i) f1(j) wrt rch(k)
  for (int i = 1; i <= 3; ++i)
    for (int j = i + 1; j <= 4; ++j)
      for (int k = 1; k <= 4; ++k) {
        T v = dfk0[i][j][k] * f1[i] * f1[j];
        if (k == i) v = v + s.fk0[i][j] * df1dc[i] * f1[j];
        if (k == j) v = v + s.fk0[i][j] * f1[i] * df1dc[j];
        s.dfdc[i][j][k] = v;
        T h = 0.0;
        if (k == i) h = s.fk0[i][j] * df1dh[i] * f1[j];
        if (k == j) h = s.fk0[i][j] * f1[i] * df1dh[j];
        s.dfdh[i][j][k] = h;
      }
}

template <class T>
inline void ipbend(State<T>& s, T* vip_out) {
  T vip = 0.0;
  ipforce(s);
  for (int i = 1; i <= 3; ++i)
    for (int j = i + 1; j <= 4; ++j) {
      T costh = s.tch[i][1] * s.tch[j][1] + s.tch[i][2] * s.tch[j][2] + s.tch[i][3] * s.tch[j][3];
      costh = costh / s.rch[i] / s.rch[j];
      T theta = acos(costh);
      T dth = theta - s.theta0[i][j];
      T kf = s.fk0[i][j] * s.f1[i] * s.f1[j];
      vip = vip + 0.5 * s.fk0[i][j] * s.f1[i] * s.f1[j] * (dth * dth);
      T termth = -1.0 / sqrt(1.0 - costh * costh);
      for (int ind = 1; ind <= 3; ++ind) {
        T dthi = -s.tch[j][ind] / s.rch[i] / s.rch[j] + costh * s.tch[i][ind] / s.rch[i] / s.rch[i];
        dthi = dthi * termth;
        T dthj = -s.tch[i][ind] / s.rch[i] / s.rch[j] + costh * s.tch[j][ind] / s.rch[j] / s.rch[j];
        dthj = dthj * termth;
        T dthc = -(dthi + dthj);
        s.pdot[s.nh[i][ind]] = s.pdot[s.nh[i][ind]] + kf * dthi * dth;
        s.pdot[s.nh[j][ind]] = s.pdot[s.nh[j][ind]] + kf * dthj * dth;
        s.pdot[s.nc[ind]] = s.pdot[s.nc[ind]] + kf * dthc * dth;
        for (int k = 1; k <= 4; ++k) {
          T dth0k = -s.dtheta0[i][j][k] * s.tch[k][ind] / s.rch[k];
          T dth0c = -dth0k;
          T d2 = dth * dth;
          s.pdot[s.nh[k][ind]] = s.pdot[s.nh[k][ind]] - 0.5 * s.tch[k][ind] * s.dfdc[i][j][k] * d2 / s.rch[k] -
                                 0.5 * s.tbh[k][ind] * s.dfdh[i][j][k] * d2 / s.rbh[k] - kf * dth0k * dth;
          s.pdot[s.nc[ind]] = s.pdot[s.nc[ind]] + 0.5 * s.tch[k][ind] * s.dfdc[i][j][k] * d2 / s.rch[k] -
                              kf * dth0c * dth;
          s.pdot[s.nhb[ind]] = s.pdot[s.nhb[ind]] + 0.5 * s.tbh[k][ind] * s.dfdh[i][j][k] * d2 / s.rbh[k];
        }
      }
    }
  // H(i)-O-H(O) harmonic bends (src/egrad_ch4oh.f:1061-1172)
  const Params& P = *s.P;
  T angh2o[5], fkh2o[5], dkdr[5], dkdx[5][4];
  for (int i = 1; i <= 4; ++i) {
    T dot = 0.0;
    for (int j = 1; j <= 3; ++j) dot = dot - s.tno[j] * s.tbh[i][j];
    T cosine = dot / (s.rno * s.rbh[i]);
    cosine = fmin(T(1.0), fmax(T(-1.0), cosine));
    angh2o[i] = acos(cosine);
  }
  for (int i = 1; i <= 4; ++i) {
    T arga = P.alph2o * (s.rbh[i] - P.r0hh);
    if (arga < 19.0) fkh2o[i] = P.fkh2oeq * (1.0 - tanh(arga));
    else fkh2o[i] = 0.0;
  }
  for (int i = 1; i <= 4; ++i) {
    T dang = angh2o[i] - P.anh2oeq;
    vip = vip + 0.5 * fkh2o[i] * dang * dang;
  }
  for (int i = 1; i <= 4; ++i) {
    T deno = cosh(P.alph2o * (s.rbh[i] - P.r0hh));
    dkdr[i] = -(P.fkh2oeq * P.alph2o) / (deno * deno);
  }
  for (int i = 1; i <= 4; ++i) {
    dkdr[i] = dkdr[i] / s.rbh[i];
    for (int j = 1; j <= 3; ++j) dkdx[i][j] = dkdr[i] * s.tbh[i][j];
  }
  for (int i = 1; i <= 4; ++i)
    for (int j = 1; j <= 3; ++j) {
      T term1 = 0.5 * sq(angh2o[i] - P.anh2oeq);
      s.pdot[s.nhb[j]] = s.pdot[s.nhb[j]] + dkdx[i][j] * term1;
      s.pdot[s.nh[i][j]] = s.pdot[s.nh[i][j]] - dkdx[i][j] * term1;
    }
  for (int i = 1; i <= 4; ++i) {
    T dstda = fkh2o[i] * (angh2o[i] - P.anh2oeq);
    T xp = s.tno[2] * s.tbh[i][3] - s.tno[3] * s.tbh[i][2];
    T yp = s.tno[3] * s.tbh[i][1] - s.tno[1] * s.tbh[i][3];
    T zp = s.tno[1] * s.tbh[i][2] - s.tno[2] * s.tbh[i][1];
    T rp = sqrt(xp * xp + yp * yp + zp * zp);
    if (rp < 1.0e-6) rp = 1.0e-6;
    T terma = dstda / (s.rbh[i] * s.rbh[i] * rp);
    T termc = dstda / (s.rno * s.rno * rp);
    T dedhi[4], dedho[4], dedo[4];
    dedhi[1] = -terma * (s.tbh[i][2] * zp - s.tbh[i][3] * yp);
    dedhi[2] = -terma * (s.tbh[i][3] * xp - s.tbh[i][1] * zp);
    dedhi[3] = -terma * (s.tbh[i][1] * yp - s.tbh[i][2] * xp);
    dedho[1] = -termc * (s.tno[2] * zp - s.tno[3] * yp);
    dedho[2] = -termc * (s.tno[3] * xp - s.tno[1] * zp);
    dedho[3] = -termc * (s.tno[1] * yp - s.tno[2] * xp);
    for (int j = 1; j <= 3; ++j) dedo[j] = -dedhi[j] - dedho[j];
    for (int j = 1; j <= 3; ++j) {
      s.pdot[s.nhb[j]] = s.pdot[s.nhb[j]] + dedo[j];
      s.pdot[s.nh[i][j]] = s.pdot[s.nh[i][j]] + dedhi[j];
      s.pdot[s.no[j]] = s.pdot[s.no[j]] + dedho[j];
    }
  }
  *vip_out = vip;
}

// egrad_ch4oh for one bead: q(3,7) column-major in bohr -> V (Eh), g (Eh/bohr);
// with geh4oh, egrad_geh4oh (src/egrad_geh4oh.f:33-67 -> pot_geh4oh).
template <class T>
inline void egrad_bead(const T* qb, T* V, T* g, bool geh4oh = false) {
  State<T> s;
  s.P = &params(geh4oh);
  const int nnc = 2, nnb = 6, nnh[5] = {0, 3, 4, 5, 1}, nno = 7;
  for (int ind = 1; ind <= 3; ++ind) {
    int icount = ind - 3;
    s.nc[ind] = 3 * nnc + icount;
    s.nhb[ind] = 3 * nnb + icount;
    s.no[ind] = 3 * nno + icount;
    for (int i = 1; i <= 4; ++i) s.nh[i][ind] = 3 * nnh[i] + icount;
  }
  for (int i = 1; i <= 21; ++i) {
    s.q[i] = qb[i - 1] * 0.52918;
    s.pdot[i] = 0.0;
  }
  coorden(s);
  switchf(s);
  refangles(s);
  T vstr, vop, vip;
  stretch(s, &vstr);
  opbend(s, &vop);
  ipbend(s, &vip);
  T en = vstr + vop + vip;
  en = en * 0.03812;
  *V = en;
  for (int i = 1; i <= 21; ++i) g[i - 1] = s.pdot[i] * 0.0201723;
}

}  // namespace ch4oh
}  // namespace orc
