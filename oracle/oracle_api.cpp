// ORACLE (test infrastructure only) -- C entry points of the CPU restatement.
#include "oracle_api.h"

#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "d3.hpp"
#include "opcount.hpp"
#include "pes_ch4h.hpp"
#include "pes_ch4oh.hpp"
#include "pes_h3.hpp"
#include "evb_fit.hpp"
#include "pes_evb.hpp"
#include "pes_qmdff.hpp"
#include "pes_water.hpp"
#include "pes_oh3.hpp"
#include "pes_brh2.hpp"
#include "philox.hpp"
#include "recross.hpp"
#include "rpmd.hpp"

namespace {

orc::StepConfig to_step(const orc_cfg* c) {
  orc::StepConfig s;
  s.natoms = c->natoms;
  s.nbeads = c->nbeads;
  s.dt = c->dt;
  s.beta = c->beta;
  s.thermostat = c->thermostat;
  s.andersen_step = c->andersen_step > 0 ? c->andersen_step : 1;
  s.pile_tau0 = c->pile_tau0;
  s.nose_q = c->nose_q;
  s.transrot = c->transrot;
  s.seed = c->seed;
  s.mass = c->mass;
  s.nm_mode = c->nm_mode;
  return s;
}

orc::qmdff::FF g_qmdff, g_qmdff2;
orc::evb::Coupling g_evb;
orc::water::Box g_water;

// Per-bead PES call, q(3,N) -> V, g(3,N).
struct BeadPES {
  int pes;
  int natoms;
  void operator()(const double* q, double* V, double* g) const {
    switch (pes) {
      case 1: orc::h3::egrad_bead<double>(q, V, g); break;
      case 2: orc::ch4h::egrad_bead<double>(q, V, g); break;
      case 3: orc::ch4oh::egrad_bead<double>(q, V, g); break;
      case 4: orc::qmdff::egrad(g_qmdff, q, V, g); break;
      case 5: orc::evb::egrad(g_qmdff, g_qmdff2, g_evb, q, V, g); break;
      case 6: *V = orc::water::egrad<double>(g_water, q, g); break;
      case 7: orc::oh3::egrad_bead<double>(q, V, g); break;
      case 8: orc::ch4oh::egrad_bead<double>(q, V, g, true); break;
      case 9: orc::brh2::egrad_bead(q, V, g); break;
      default: *V = NAN; for (int x = 0; x < 3 * natoms; ++x) g[x] = NAN; break;
    }
  }
};

}  // namespace

extern "C" {

void orc_water_set(int nwater, int periodic, const double* len, double coul_cut, int zahn, double zahn_a,
                   double zahn_par) {
  orc::water::Box& b = g_water;
  b.nwater = nwater;
  b.periodic = periodic;
  for (int k = 0; k < 3; ++k) b.len[k] = len ? len[k] : 0.0;
  b.coul_cut = coul_cut;
  b.zahn = zahn;
  b.zahn_a = zahn_a;
  b.zahn_par = zahn_par;
}

void orc_qmdff_set_periodic(const double* box_ang, double coul_cut_ang, double vdw_cut_ang, double* cuts) {
  orc::qmdff::set_periodic(g_qmdff, box_ang, coul_cut_ang, vdw_cut_ang);
  if (cuts) {
    cuts[0] = g_qmdff.coul_cut;
    cuts[1] = g_qmdff.vdw_cut;
    cuts[2] = g_qmdff.zahn_a;
    cuts[3] = g_qmdff.zahn_par;
  }
}

int orc_qmdff_egrad_virial(const double* q, int nbeads, const double* box, double* V, double* g, double* vir) {
  if (!g_qmdff.periodic && box) return -1;
  orc::qmdff::FF ff = g_qmdff;
  const size_t n3 = (size_t)3 * ff.n;
  for (int b = 0; b < nbeads; ++b) {
    if (box)
      for (int k = 0; k < 3; ++k) {
        ff.len[k] = box[3 * (size_t)b + k];
        ff.half[k] = ff.len[k] * 0.5;
      }
    double w = 0.0;
    ff.vir = &w;
    orc::qmdff::egrad(ff, &q[b * n3], &V[b], &g[b * n3]);
    vir[b] = w;
  }
  return 0;
}

int orc_run_npt(const orc_cfg* cf, int ntraj, uint32_t traj0, int istep0, int nsteps, double* q, double* p,
                double* f, double* epot, int* status, double* box, double* press, double pressure, double compress,
                double taupres, int nthreads) {
  if (cf->pes != 4 || !g_qmdff.periodic || !box || !press) return -1;
  orc::StepConfig s = to_step(cf);
  orc::NptConfig np;
  np.pressure = pressure;
  np.compress = compress;
  np.taupres = taupres;
  const size_t per = (size_t)3 * cf->natoms * cf->nbeads;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int t = 0; t < ntraj; ++t) {
    orc::qmdff::FF ff = g_qmdff;  // this trajectory's box
    double w = 0.0;
    ff.vir = &w;
    double* L = &box[3 * (size_t)t];
    auto pes = [&](const double* qb, double* V, double* g) {
      for (int k = 0; k < 3; ++k) {
        ff.len[k] = L[k];
        ff.half[k] = L[k] * 0.5;
      }
      orc::qmdff::egrad(ff, qb, V, g);
    };
    int st = 0;
    double e = 0.0;
    for (int n = 1; n <= nsteps; ++n)
      st |= orc::verlet_step_npt(s, np, traj0 + t, istep0 + n, &q[t * per], &p[t * per], &f[t * per], &e, pes, L,
                                 &press[t], &w);
    if (epot) epot[t] = e;
    if (status) status[t] |= st;
  }
  return 0;
}

void orc_qmdff_set2(const orc_qmdff_def* d) {
  orc::qmdff::FF keep = g_qmdff;
  orc_qmdff_set(d);
  g_qmdff2 = g_qmdff;
  g_qmdff = keep;
}

void orc_evb_set(int basis, const double* par) {
  g_evb.basis = basis;
  double* dst[10] = {&g_evb.a, &g_evb.b, &g_evb.c, &g_evb.d, &g_evb.e, &g_evb.f, &g_evb.g, &g_evb.h, &g_evb.m, &g_evb.n};
  for (int k = 0; k < 10; ++k) *dst[k] = par[k];
}

void orc_qmdff_set(const orc_qmdff_def* d) {
  orc::qmdff::FF& f = g_qmdff;
  f = orc::qmdff::FF();
  f.n = d->natoms;
  f.at.assign(d->at, d->at + f.n);
  f.q.assign(d->q, d->q + f.n);
  f.rad.assign(d->rad, d->rad + f.n);
  f.nbond = d->nbond;
  f.nangl = d->nangl;
  f.ntors = d->ntors;
  f.nnci = d->nnci;
  f.bond.assign(d->bond, d->bond + 2 * f.nbond);
  f.vbond.assign(d->vbond, d->vbond + 3 * f.nbond);
  f.angl.assign(d->angl, d->angl + 3 * f.nangl);
  f.vangl.assign(d->vangl, d->vangl + 2 * f.nangl);
  f.tors.assign(d->tors, d->tors + 6 * f.ntors);
  f.vtors.assign(d->vtors, d->vtors + 14 * f.ntors);
  f.nci.assign(d->nci, d->nci + 3 * f.nnci);
  f.pR0.assign(d->pR0, d->pR0 + f.nnci);
  f.pC6.assign(d->pC6, d->pC6 + f.nnci);
  f.pSr42.assign(d->pSr42, d->pSr42 + f.nnci);
  f.pZab.assign(d->pZab, d->pZab + f.nnci);
  f.pAlpha.assign(d->pAlpha, d->pAlpha + f.nnci);
  f.nhb = d->nhb;
  if (f.nhb > 0) {
    f.hb.assign(d->hb, d->hb + 3 * f.nhb);
    f.vhb.assign(d->vhb, d->vhb + 2 * f.nhb);
  }
  for (int i = 0; i < 7; ++i) {
    f.eps1[i] = d->eps1[i];
    f.eps2[i] = d->eps2[i];
  }
  f.coul_cut = d->coul_cut;
  f.zahn = d->zahn != 0;
  f.zahn_a = d->zahn_a;
  f.zahn_par = d->zahn_par;
  f.e_zero = d->e_zero;
}

void orc_philox4x32_10(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
  orc::Philox4 r = orc::philox4x32_10(ctr, k0, k1);
  for (int i = 0; i < 4; ++i) out[i] = r.v[i];
}

void orc_normal_pair(uint32_t seed, uint32_t traj, uint32_t pair, uint32_t bead, uint32_t step,
                     uint32_t tag, double out[2]) {
  orc::normal_pair(seed, traj, pair, bead, step, tag, &out[0], &out[1]);
}

void orc_h3_pote(const double R[3], double* V, double dV[3]) { orc::h3::pote<double>(R, V, dV); }

void orc_egrad_h3(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info) {
  if (info) *info = 0;
  for (int k = 0; k < nbeads; ++k)
    orc::h3::egrad_bead<double>(&q[(size_t)k * 3 * natoms], &V[k], &dVdq[(size_t)k * 3 * natoms]);
}

void orc_egrad(int pes, const double* q, int natoms, int nbeads, double* V, double* dVdq) {
  BeadPES f{pes, natoms};
  for (int k = 0; k < nbeads; ++k)
    f(&q[(size_t)k * 3 * natoms], &V[k], &dVdq[(size_t)k * 3 * natoms]);
}

void orc_cos_transform(double* x, int P) { orc::caracal_cos_transform(x, P); }

int orc_transrot(const orc_cfg* cf, const double* q, double* p) {
  orc::StepConfig s = to_step(cf);
  return orc::transrot(s, q, p);
}

void orc_init_positions(const orc_cfg* cf, int ntraj, uint32_t traj0, const double* q0,
                        double sigma, double* q) {
  const int N = cf->natoms, P = cf->nbeads;
  std::vector<double> z(3 * N);
  for (int t = 0; t < ntraj; ++t)
    for (int k = 0; k < P; ++k) {
      orc::normals_bead(cf->seed, traj0 + t, (uint32_t)k, 0, orc::TAG_BEAD_JITTER, 3 * N, z.data());
      double* qq = &q[((size_t)t * P + k) * 3 * N];
      for (int x = 0; x < 3 * N; ++x) qq[x] = q0[x] + sigma * z[x];
    }
}

void orc_init_momenta_draw(const orc_cfg* cf, int ntraj, uint32_t traj0, uint32_t draw, double* p) {
  orc::StepConfig s = to_step(cf);
  const size_t per = (size_t)3 * cf->natoms * cf->nbeads;
  for (int t = 0; t < ntraj; ++t) orc::andersen(s, traj0 + t, draw, orc::TAG_INIT_MOMENTA, &p[t * per]);
}

void orc_init_momenta(const orc_cfg* cf, int ntraj, uint32_t traj0, double* p) {
  orc_init_momenta_draw(cf, ntraj, traj0, 0u, p);
}

int orc_init_forces(const orc_cfg* cf, int ntraj, const double* q, double* f, double* epot) {
  BeadPES pes{cf->pes, cf->natoms};
  const int n3 = 3 * cf->natoms, P = cf->nbeads;
  for (int t = 0; t < ntraj; ++t) {
    double e = 0.0;
    for (int k = 0; k < P; ++k) {
      double v;
      size_t off = ((size_t)t * P + k) * n3;
      pes(&q[off], &v, &f[off]);
      e = e + v;
    }
    if (epot) epot[t] = e;
  }
  return 0;
}

int orc_run(const orc_cfg* cf, int ntraj, uint32_t traj0, int istep0, int nsteps, double* q,
            double* p, double* f, double* epot, int* status, int nthreads, double* vnh) {
  if (cf->thermostat == 2 && !vnh) return -1;
  orc::StepConfig s = to_step(cf);
  BeadPES pes{cf->pes, cf->natoms};
  const size_t per = (size_t)3 * cf->natoms * cf->nbeads;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int t = 0; t < ntraj; ++t) {
    int st = 0;
    double e = 0.0;
    for (int n = 1; n <= nsteps; ++n)
      st |= orc::verlet_step(s, traj0 + t, istep0 + n, &q[t * per], &p[t * per], &f[t * per], &e, pes,
                             vnh ? &vnh[4 * (size_t)t] : nullptr);
    if (epot) epot[t] = e;
    if (status) status[t] |= st;
  }
  return 0;
}

void orc_nhc_half(const orc_cfg* cf, double* vnh, double* p) {
  orc::StepConfig s = to_step(cf);
  orc::nhc_half(s, vnh, p);
}

static orc::XiDef to_xi(const orc_xidef* x) {
  orc::XiDef d;
  d.nreac1 = x->nreac1;
  d.nreac2 = x->nreac2;
  for (int i = 0; i < 8; ++i) {
    d.reac1[i] = x->reac1[i];
    d.reac2[i] = x->reac2[i];
  }
  d.form[0] = x->form[0];
  d.form[1] = x->form[1];
  d.brk[0] = x->brk[0];
  d.brk[1] = x->brk[1];
  d.form_ref = x->form_ref;
  d.break_ref = x->break_ref;
  d.r_inf = x->r_inf;
  d.xi_ideal = x->xi_ideal;
  return d;
}

int orc_run_parent(const orc_cfg* cf, const orc_xidef* xd, int ntraj, uint32_t traj0, int istep0, int nsteps,
                   double* q, double* p, double* f, double* epot, int* status, double* dxi, double* vnh) {
  if (cf->thermostat == 2 && !vnh) return -1;
  orc::StepConfig s = to_step(cf);
  s.transrot = 0;
  const orc::XiDef x = to_xi(xd);
  BeadPES pes{cf->pes, cf->natoms};
  const int n3 = 3 * cf->natoms;
  const size_t per = (size_t)n3 * cf->nbeads;
  for (int t = 0; t < ntraj; ++t) {
    double* d = &dxi[(size_t)t * n3];
    bool zero = true;
    for (int k = 0; k < n3; ++k) zero = zero && d[k] == 0.0;
    if (zero) {
      std::vector<double> c(n3);
      orc::centroid(cf->natoms, cf->nbeads, &q[t * per], c.data());
      orc::calc_xi_mode2(x, cf->natoms, c.data(), cf->mass, d);
    }
    int st = 0;
    double e = 0.0;
    for (int n = 1; n <= nsteps; ++n)
      st |= orc::parent_step(s, x, traj0 + t, istep0 + n, &q[t * per], &p[t * per], &f[t * per], &e, d, pes,
                             vnh ? &vnh[4 * (size_t)t] : nullptr);
    if (epot) epot[t] = e;
    if (status) status[t] |= st;
  }
  return 0;
}

// Umbrella sampling windows: trajectory t is biased towards centers[t] with
// force constant kforce[t] (Eh); with sampling set, the xi of every step is
// added to xsum, xsum2 and (nbins > 0) the histogram hist[t][nbins] over
// [lo, hi).  Same step as orc_run otherwise.
int orc_run_umbrella(const orc_cfg* cf, const orc_xidef* xd, int ntraj, uint32_t traj0, int istep0, int nsteps,
                     const double* centers, const double* kforce, double* q, double* p, double* f, double* epot,
                     int* status, double* vnh, int sampling, double* xsum, double* xsum2, int nbins, double lo,
                     double hi, double* hist) {
  if (cf->thermostat == 2 && !vnh) return -1;
  orc::StepConfig s = to_step(cf);
  const orc::XiDef x = to_xi(xd);
  BeadPES pes{cf->pes, cf->natoms};
  const size_t per = (size_t)3 * cf->natoms * cf->nbeads;
  for (int t = 0; t < ntraj; ++t) {
    int st = 0;
    double e = 0.0;
    for (int n = 1; n <= nsteps; ++n) {
      double xi = 0.0;
      auto bias = [&](const double* qq, double* ff) { xi = orc::umbrella_bias(s, x, centers[t], kforce[t], qq, ff); };
      st |= orc::verlet_step(s, traj0 + t, istep0 + n, &q[t * per], &p[t * per], &f[t * per], &e, pes,
                             vnh ? &vnh[4 * (size_t)t] : nullptr, bias);
      if (sampling) {
        xsum[t] = xsum[t] + xi;
        xsum2[t] = xsum2[t] + xi * xi;
        if (nbins > 0) {
          const double u = (xi - lo) / (hi - lo) * nbins;
          if (u >= 0.0 && u < nbins) hist[(size_t)t * nbins + (int)u] += 1.0;
        }
      }
    }
    if (epot) epot[t] = e;
    if (status) status[t] |= st;
  }
  return 0;
}

double orc_umbrella_bias(const orc_cfg* cf, const orc_xidef* xd, double xi0, double kforce, const double* q,
                         double* f) {
  return orc::umbrella_bias(to_step(cf), to_xi(xd), xi0, kforce, q, f);
}

double orc_calc_xi_umbrella(const orc_xidef* xd, int natoms, const double* coords, const double* mass, double* dxi,
                            double* d2xi) {
  return orc::calc_xi_mode1(to_xi(xd), natoms, coords, mass, dxi, d2xi);
}

double orc_calc_xi(const orc_xidef* xd, int natoms, const double* coords, const double* mass,
                   double* dxi) {
  return orc::calc_xi_mode2(to_xi(xd), natoms, coords, mass, dxi);
}

int orc_recross_children(const orc_cfg* cf, const orc_xidef* xd, int ntraj, uint32_t traj0,
                         const double* q_parent, int nsteps, double* num, double* denom,
                         double* w_out, double* q_out, double* p_out, int nthreads) {
  orc::StepConfig s = to_step(cf);
  orc::XiDef x = to_xi(xd);
  BeadPES pes{cf->pes, cf->natoms};
  const size_t per = (size_t)3 * cf->natoms * cf->nbeads;
  std::vector<double> w(ntraj);
  std::vector<unsigned char> side((size_t)ntraj * nsteps), pos(ntraj);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int t = 0; t < ntraj; ++t) {
    std::vector<double> q(per), p(per), f(per);
    bool vp = false;
    w[t] = orc::recross_child(s, x, traj0 + (uint32_t)(t & ~1), (t & 1) != 0, q_parent, nsteps, q.data(),
                              p.data(), f.data(), &side[(size_t)t * nsteps], &vp, pes);
    pos[t] = vp ? 1 : 0;
    if (q_out)
      for (size_t i = 0; i < per; ++i) q_out[t * per + i] = q[i];
    if (p_out)
      for (size_t i = 0; i < per; ++i) p_out[t * per + i] = p[i];
  }
  double den = 0.0;
  for (int t = 0; t < ntraj; ++t)
    if (pos[t]) den = den + w[t];
  if (denom) *denom = den;
  for (int st = 0; st < nsteps; ++st) {
    double acc = 0.0;
    for (int t = 0; t < ntraj; ++t)
      if (side[(size_t)t * nsteps + st]) acc = acc + w[t];
    num[st] = acc;
  }
  if (w_out)
    for (int t = 0; t < ntraj; ++t) w_out[t] = w[t];
  return 0;
}

void orc_pes_opcount(int pes, const double* q, uint64_t out[14]) {
  orc::tally().reset();
  if (pes == 1) {
    orc::OC qq[9], V, g[9];
    for (int x = 0; x < 9; ++x) qq[x] = orc::OC(q[x]);
    orc::h3::egrad_bead<orc::OC>(qq, &V, g);
  } else if (pes == 2) {
    orc::OC qq[18], V, g[18];
    for (int x = 0; x < 18; ++x) qq[x] = orc::OC(q[x]);
    orc::ch4h::egrad_bead<orc::OC>(qq, &V, g);
  } else if (pes == 3 || pes == 8) {
    orc::OC qq[21], V, g[21];
    for (int x = 0; x < 21; ++x) qq[x] = orc::OC(q[x]);
    orc::ch4oh::egrad_bead<orc::OC>(qq, &V, g, pes == 8);
  } else if (pes == 4) {
    const int n3 = 3 * g_qmdff.n;
    std::vector<orc::OC> qq((size_t)n3), g((size_t)n3);
    orc::OC V;
    for (int x = 0; x < n3; ++x) qq[(size_t)x] = orc::OC(q[x]);
    orc::qmdff::egrad<orc::OC>(g_qmdff, qq.data(), &V, g.data());
  } else if (pes == 7) {
    orc::OC qq[12], V, g[12];
    for (int x = 0; x < 12; ++x) qq[x] = orc::OC(q[x]);
    orc::oh3::egrad_bead<orc::OC>(qq, &V, g);
  } else if (pes == 6) {
    const int n3 = 9 * g_water.nwater;
    std::vector<orc::OC> qq((size_t)n3), g((size_t)n3);
    for (int x = 0; x < n3; ++x) qq[(size_t)x] = orc::OC(q[x]);
    orc::water::egrad<orc::OC>(g_water, qq.data(), g.data());
  }
  const orc::OpTally& t = orc::tally();
  uint64_t v[14] = {t.add, t.mul, t.div,  t.sqrt, t.exp, t.log,  t.pow,
                    t.sin, t.cos, t.acos, t.erf,  t.cmp, t.tanh, t.cosh};
  for (int i = 0; i < 14; ++i) out[i] = v[i];
}

int orc_evb_fit(int basis, const double* x, int npar, int m, const double* e1, const double* e2,
                const double* eref, double* fvec, double* fjac) {
  if (basis < 1 || basis > 8) return -1;
  orc::evbfit::residual(basis, x, m, e1, e2, eref, fvec);
  if (fjac) orc::evbfit::fdjac2(basis, std::vector<double>(x, x + npar), m, e1, e2, eref, fvec, 0.0, fjac);
  return 0;
}

}  // extern "C"

extern "C" void orc_d3_pair_c6(const double* pars, int nlines, int n, const int* at, const double* xyz,
                               const double* rcov, double* c6xy, double* cn) {
  orc::D3Ref d;
  orc::copyc6(pars, nlines, d);
  orc::pair_c6(d, n, at, xyz, rcov, c6xy, cn);
}
