/* ORACLE (test infrastructure only) -- C entry points of the CPU restatement.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library, and only as the checker.  Arrays are Fortran column-major
 * q(3, natoms, nbeads) per trajectory, trajectories outermost. */
#ifndef CARACAL_ORACLE_API_H
#define CARACAL_ORACLE_API_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_cfg {
  int pes;            /* 1 H3 (BKMP2), 2 CH4H, 3 CH4OH, 4 QMDFF (orc_qmdff_set), 5 dE-EVB of two QMDFFs,
                         6 flexible SPC water box (orc_water_set), 7 OH + H2 (ANA_OH3), 8 GeH4 + OH
                         (ANA_GEH4OH), 9 Br + H2 (ANA_BRH2) */
  int natoms;
  int nbeads;
  int thermostat;     /* 0 none, 1 Andersen, 2 Nose-Hoover chain, 3 PILE */
  int andersen_step;
  int transrot;       /* 1: remove COM translation/rotation every step */
  uint32_t seed;
  double dt;          /* a.u. */
  double beta;        /* a.u. */
  double pile_tau0;   /* a.u. */
  const double* mass; /* natoms, a.u. */
  double nose_q;      /* a.u.: NOSE_Q (time steps) x dt */
  int nm_mode;        /* 0: Caracal's cosine transform; 1: orthonormal real normal modes */
} orc_cfg;

void orc_philox4x32_10(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]);
void orc_normal_pair(uint32_t seed, uint32_t traj, uint32_t pair, uint32_t bead, uint32_t step,
                     uint32_t tag, double out[2]);
void orc_h3_pote(const double R[3], double* V, double dV[3]);
/* egrad_h3(q, Natoms, Nbeads, V, dVdq, info) of src/egrad_h3.f:29 */
void orc_egrad_h3(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info);
/* any PES (1 = H3, 2 = CH4H): q(3,natoms,nbeads) -> V(nbeads), dVdq */
void orc_egrad(int pes, const double* q, int natoms, int nbeads, double* V, double* dVdq);
void orc_cos_transform(double* x, int P);
int orc_transrot(const orc_cfg* cf, const double* q, double* p);
/* bead jitter: q[t] = q0 + sigma * N(0,1) (tag 4, step 0) */
void orc_init_positions(const orc_cfg* cf, int ntraj, uint32_t traj0, const double* q0,
                        double sigma, double* q);
/* mdinit: Andersen draw at step 0 (tag 0) */
void orc_init_momenta(const orc_cfg* cf, int ntraj, uint32_t traj0, double* p);
/* prepare's D3 pair C6 (copyc6 + ncoord_qmdff + getc6) of n atoms at xyz(3, n) bohr:
 * c6xy (n x n), cn (n) */
void orc_d3_pair_c6(const double* pars, int nlines, int n, const int* at, const double* xyz,
                    const double* rcov, double* c6xy, double* cn);
/* mdinit's Andersen draw number `draw` (Gaussian stream counter; 0 as above) */
void orc_init_momenta_draw(const orc_cfg* cf, int ntraj, uint32_t traj0, uint32_t draw, double* p);
/* mdinit: forces of the initial positions; epot[t] = sum over beads */
int orc_init_forces(const orc_cfg* cf, int ntraj, const double* q, double* f, double* epot);
/* nsteps verlet steps (istep0+1 .. istep0+nsteps) of ntraj trajectories;
 * status[t] ORs the per-step status bits; nthreads <= 0 uses all cores.
 * vnh[4 * ntraj]: Nose-Hoover chain velocities (in/out; NULL unless
 * thermostat 2). */
int orc_run(const orc_cfg* cf, int ntraj, uint32_t traj0, int istep0, int nsteps, double* q,
            double* p, double* f, double* epot, int* status, int nthreads, double* vnh);
/* One nhc call (src/nhc.f90) on one trajectory's p(3,natoms,nbeads); vnh[4] in/out. */
void orc_nhc_half(const orc_cfg* cf, double* vnh, double* p);
/* QMDFF definition (0-based atoms); per-NCI-pair R0, C6, sr42, zab, alpha. */
typedef struct orc_qmdff_def {
  int natoms;
  const int* at;
  const double* q;
  const double* rad;  /* covalent radius per atom, bohr */
  int nbond, nangl, ntors, nnci;
  const int* bond;    /* 2 per bond */
  const double* vbond;
  const int* angl;    /* 3 per angle, centre first */
  const double* vangl;
  const int* tors;    /* 6 per torsion */
  const double* vtors;/* 14 per torsion */
  const int* nci;     /* 3 per pair */
  const double *pR0, *pC6, *pSr42, *pZab, *pAlpha;
  int nhb;
  const int* hb;      /* 3 per triple: A, B, H (0-based) */
  const double* vhb;  /* 2 per triple */
  double eps1[7], eps2[7];
  double coul_cut;
  int zahn;
  double zahn_a, zahn_par, e_zero;
} orc_qmdff_def;

/* Sets the force field used by PES id 4 (QMDFF) in all oracle entry points. */
void orc_qmdff_set(const orc_qmdff_def* d);
/* set_periodic for the current force field: box edges and cutoffs in
 * Angstrom; cuts (may be NULL) receives coul_cut, vdw_cut, zahn_a, zahn_par
 * as set (bohr). */
void orc_qmdff_set_periodic(const double* box_ang, double coul_cut_ang, double vdw_cut_ang, double* cuts);
/* The current force field on nbeads beads q(3, n, nbeads): V, g and each
 * bead's virial trace vir[b] (the reference's vir_ten terms), the box of
 * bead b box[3 b .. 3 b + 2] (bohr) where box is not NULL (the force field
 * must be periodic).  Returns 0, or -1 for a box without set_periodic. */
int orc_qmdff_egrad_virial(const double* q, int nbeads, const double* box, double* V, double* g, double* vir);
/* orc_run with the Berendsen barostat (PES 4, periodic): box[3 t ..] (bohr)
 * per trajectory in and out, press[t] the pressure of the last step (a.u.);
 * pressure (a.u.), compress and taupres as mdinit sets them. */
int orc_run_npt(const orc_cfg* cf, int ntraj, uint32_t traj0, int istep0, int nsteps, double* q, double* p,
                double* f, double* epot, int* status, double* box, double* press, double pressure, double compress,
                double taupres, int nthreads);
/* The second force field and the coupling of PES id 5 (dE-EVB of the two):
 * basis 0..7 = const, 1g, 2g, 3g, sp, sd, sd2, sp2d; par = offa..offh, offm, offn. */
void orc_qmdff_set2(const orc_qmdff_def* d);
/* PES 6: Caracal's flexible SPC water box (src/egrad_water.f90): nwater
 * molecules O, H, H; periodic boundaries with box lengths len[3] (bohr) and
 * the Coulomb cutoff, Zahn form if zahn. */
void orc_water_set(int nwater, int periodic, const double* len, double coul_cut, int zahn, double zahn_a,
                   double zahn_par);
void orc_evb_set(int basis, const double par[10]);

/* BIMOLEC reaction coordinate of Caracal's recrossing (calc_xi mode 2). */
typedef struct orc_xidef {
  int nreac1, reac1[8];   /* 0-based atom indices of reactant 1 */
  int nreac2, reac2[8];   /* 0-based atom indices of reactant 2 */
  int form[2], brk[2];    /* 0-based atoms of the forming and the breaking bond */
  double form_ref, break_ref, r_inf, xi_ideal;
} orc_xidef;

int orc_run_umbrella(const orc_cfg* cf, const orc_xidef* xd, int ntraj, uint32_t traj0, int istep0, int nsteps,
                     const double* centers, const double* kforce, double* q, double* p, double* f, double* epot,
                     int* status, double* vnh, int sampling, double* xsum, double* xsum2, int nbins, double lo,
                     double hi, double* hist);
double orc_umbrella_bias(const orc_cfg* cf, const orc_xidef* xd, double xi0, double kforce, const double* q,
                         double* f);
double orc_calc_xi_umbrella(const orc_xidef* xd, int natoms, const double* coords, const double* mass, double* dxi,
                            double* d2xi);
double orc_calc_xi(const orc_xidef* xd, int natoms, const double* coords, const double* mass,
                   double* dxi);
/* ntraj recrossing children (pairs 2i, 2i+1 share momenta with opposite
 * signs, keyed by traj0 + 2i) from the parent ring polymer q_parent(3,N,P):
 * num[s] = sum over children of w * [xi > 0 after step s+1], denom = sum of
 * w over children with vs > 0, w = vs/fs; q_out/p_out get the final states
 * (may be NULL). */
int orc_recross_children(const orc_cfg* cf, const orc_xidef* xd, int ntraj, uint32_t traj0,
                         const double* q_parent, int nsteps, double* num, double* denom,
                         double* w_out, double* q_out, double* p_out, int nthreads);

/* nsteps steps of ntraj constrained parent trajectories (verlet with
 * constrain = 1: SHAKE/RATTLE on the xi(centroid) = 0 surface, no transrot);
 * dxi[ntraj * 3 * natoms] in/out is each parent's dxi_act (zeros: computed
 * from the current centroid first).  status bit 4: SHAKE did not converge. */
int orc_run_parent(const orc_cfg* cf, const orc_xidef* xd, int ntraj, uint32_t traj0, int istep0, int nsteps,
                   double* q, double* p, double* f, double* epot, int* status, double* dxi, double* vnh);

/* dE-EVB coupling fit (src/lm_de_func.f90, src/lm_good.f fdjac2): fvec[m]
 * and, if fjac is not NULL, the forward-difference Jacobian fjac[npar][m];
 * basis 1..8 = 1g, 2g, 3g, sp, sd, sd2, sp2d, sp2d3. */
int orc_evb_fit(int basis, const double* x, int npar, int m, const double* e1, const double* e2,
                const double* eref, double* fvec, double* fjac);

/* algorithmic operation tallies (add, mul, div, sqrt, exp, log, pow, sin, cos,
 * acos, erf, cmp, tanh, cosh) of one PES evaluation of one bead at geometry q. */
void orc_pes_opcount(int pes, const double* q, uint64_t out[14]);

#ifdef __cplusplus
}
#endif
#endif
