/*
 * caracal_gb300.h -- C-ABI of the GB300-native RPMD engine.
 *
 * A drop-in for the hot path of Caracal's `dynamic` / `calc_rate` programs:
 * the per-bead PES gradient calls and the ring-polymer `verlet` step.  Every
 * entry point takes plain pointers and sizes and returns an int status
 * (CR_OK = 0, > 0 error; nothing in this library calls exit()).  Host arrays
 * use Caracal's Fortran column-major layout q(3, natoms, nbeads) per
 * trajectory, with trajectories outermost: element (d, i, k, t) sits at
 * d + 3*(i + natoms*(k + nbeads*t)).  Units are atomic units (bohr, Hartree,
 * electron masses), as inside Caracal.
 *
 * Each engine owns one CUDA stream and its device memory on the device that
 * is current when it is created; calls on one engine are not thread-safe,
 * different engines are independent.
 */
#ifndef CARACAL_GB300_H
#define CARACAL_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define CR_OK 0
#define CR_ERR_ARG 1          /* invalid argument or configuration */
#define CR_ERR_CUDA 2         /* a CUDA runtime call failed */
#define CR_ERR_NO_DEVICE 3    /* no CUDA device visible */
#define CR_ERR_UNSUPPORTED 4  /* valid in Caracal, not provided by this engine */
#define CR_ERR_TRAJECTORY 5   /* a trajectory went non-finite (Caracal: fatal) */
#define CR_ERR_IO 6           /* file could not be read or parsed */

/* per-trajectory status bits (cr_engine_get_state) */
#define CR_TRAJ_NONFINITE 1        /* a coordinate became NaN/Inf (src/verlet.f90:1256-1275) */
#define CR_TRAJ_SINGULAR_INERTIA 2 /* transrot could not invert the inertia tensor */
#define CR_TRAJ_SHAKE_FAILED 4     /* constrained parent: SHAKE did not converge (src/verlet.f90:751-756) */

/* ---- potentials (Caracal keyword PES) ----------------------------------- */
#define CR_PES_H3 1      /* ANA_H3: BKMP2, src/egrad_h3.f */
#define CR_PES_CH4H 2    /* ANA_CH4H: src/egrad_ch4h.f + src/util_ch4h.f */
#define CR_PES_CH4OH 3   /* ANA_CH4OH: src/egrad_ch4oh.f + src/util_ch4oh.f */
#define CR_PES_QMDFF 4   /* QMDFF: src/ff_eg.f90, ff_nonb.f90, ff_hb.f90 */
#define CR_PES_EVB 5     /* dE-EVB of two QMDFFs: src/gradient.f90:361-386, 1228-1304 */
#define CR_PES_WATER 6   /* flexible SPC water box: src/egrad_water.f90, src/water_init.f90 */
#define CR_PES_OH3 7     /* ANA_OH3: OH + H2 (Schatz-Elgersma), src/egrad_oh3.f */
#define CR_PES_GEH4OH 8  /* ANA_GEH4OH: GeH4 + OH, src/egrad_geh4oh.f + src/util_geh4oh.f */
#define CR_PES_BRH2 9    /* ANA_BRH2: Br + H2 (DIM-3C), src/egrad_brh2.f */

/* ---- thermostats (Caracal keyword THERMOSTAT) ---------------------------- */
#define CR_THERMO_NONE 0      /* NVE */
#define CR_THERMO_ANDERSEN 1  /* src/andersen.f90 */
#define CR_THERMO_NHC 2       /* Nose-Hoover chain, src/nhc.f90 */
#define CR_THERMO_PILE 3      /* PILE-L, new (Ceriotti et al. 2010) */

/* ---- precision forms ------------------------------------------------------ */
#define CR_PREC_FP64 0   /* plain form: everything in FP64 */
#define CR_PREC_MIXED 1  /* PES arithmetic in FP32; q, p, propagator, thermostat in FP64 */

typedef struct cr_config {
  int pes;            /* CR_PES_* */
  int natoms;         /* must match the PES (H3 and BrH2: 3, CH4H: 6, CH4OH and GeH4OH: 7, OH3: 4, QMDFF: the force field's n) */
  int nbeads;         /* 1..128 (RPMD_BEADS) */
  int ntraj;          /* independent trajectories in this engine */
  int thermostat;     /* CR_THERMO_* */
  int andersen_step;  /* ANDERSEN_STEP (Caracal default 70) */
  int transrot;       /* 1: remove COM translation/rotation each step (dynamic.x); 0: off (recrossing children) */
  int precision;      /* CR_PREC_* */
  unsigned int seed;  /* Gaussian stream key */
  unsigned int traj0; /* global index of this engine's first trajectory (stream key) */
  double dt;          /* time step, a.u. (Caracal: DELTAT[fs] / 2.41888428E-2 as REAL(4)) */
  double beta;        /* 1/(k_B T), a.u., k_B = 0.316679e-5 Eh/K */
  double pile_tau0;   /* PILE centroid time constant, a.u. */
  const double* mass; /* natoms masses, a.u. (amu / 5.485799095e-4) */
  double nose_q;      /* NHC chain time, a.u.: NOSE_Q (in time steps) x dt (src/dynamic.f90:578) */
  int nm_mode;        /* normal-mode transform of the free ring polymer: 0 = Caracal's (rfft/irfft
                         both keep sqrt(1/P) Re DFT, src/rfft.f90, src/irfft.f90: every step projects
                         onto bead-reflection-symmetric configurations); 1 = orthonormal real normal
                         modes (standard RPMD; not Caracal's code path, an engine option) */
} cr_config;

/* ---- flexible SPC water box (water_spc: src/egrad_water.f90:36-333) -------
 * nwater molecules with atoms ordered O, H, H (src/water_init.f90:53-72) and
 * Caracal's fixed parameters (src/water_init.f90:74-103): Morse OH, harmonic
 * HH, bond-angle and bond-bond couplings, point charges -0.82 / 0.41 e,
 * Coulomb (or the Zahn form) between molecules and LJ 12-6 where the pair's
 * first atom is an oxygen.  With periodic = 1 every distance vector takes
 * the minimum image of the orthorhombic box (src/box_image.f90) and pairs at
 * r >= coul_cut are skipped (src/set_periodic.f90 sets coul_cut and, for
 * Zahn, zahn_a = 0.2 bohr and zahn_par from the cutoff). */
typedef struct cr_water_def {
  int nwater;
  int periodic;
  double box[3];     /* box lengths, bohr */
  double coul_cut;   /* bohr */
  int zahn;
  double zahn_a, zahn_par;
} cr_water_def;
typedef struct cr_water cr_water;
int cr_water_create(const cr_water_def* def, cr_water** out);
int cr_water_destroy(cr_water* w);
int cr_water_natoms(const cr_water* w);
/* Energies V(nbeads) and gradients dVdq(3, natoms, nbeads) of host arrays
 * q(3, natoms, nbeads), precision CR_PREC_FP64 or CR_PREC_MIXED. */
int cr_water_egrad(const cr_water* w, const double* q, int nbeads, double* V, double* dVdq, int precision);

typedef struct cr_engine cr_engine;

/* Human-readable text for a status code, and the detail of the last error
 * raised on this thread (copied into buf, NUL-terminated). */
const char* cr_error_string(int code);
int cr_last_error_detail(char* buf, int len);

int cr_device_count(int* n);

/* ---- PES gradient entry points --------------------------------------------
 * Replaces `subroutine egrad_h3(q,Natoms,Nbeads,V,dVdq,info)`
 * (src/egrad_h3.f:29-35; called from src/gradient.f90:172-200): q(3,natoms,nbeads)
 * in bohr -> V(nbeads) in Hartree, dVdq(3,natoms,nbeads) in Hartree/bohr, info = 0.
 * Host pointers; all beads are evaluated in one device launch (FP64). */
int cr_egrad_h3(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info);

/* No counterpart in Caracal.  The same BKMP2 gradient as cr_egrad_h3 (FP64,
 * same arguments) for callers that cannot allocate device memory: an MD loop
 * calling the PES every step cannot pay the device-wide synchronisation of
 * cudaMalloc/cudaFree per call, and a host whose device memory belongs to its
 * own pre-sized pool may not allocate outside it.  Stages through one fixed
 * file-scope device array (2.49 MB per device, held until exit) and allocates
 * nothing.  At most 16384 beads per call (more: CR_ERR_ARG).  All calls share
 * that array, so calls that overlap on the GPU race; serialise them.  The
 * first call on a device resolves the array's address (set-up), so make it
 * before any stream capture.  Runs on the legacy default stream with
 * blocking copies: a call waits for, and holds up, work on every blocking
 * stream of the device, and returns with the results on the host. */
int cr_egrad_h3_noalloc(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info);

/* Same surface on device-resident arrays with an explicit precision form
 * (CR_PREC_*); stream may be 0.  npts = number of (natoms=3) geometries. */
int cr_egrad_h3_device(const double* d_q, int npts, double* d_V, double* d_dVdq, int precision,
                       void* stream);

/* Replaces `subroutine egrad_ch4h(q,Natoms,Nbeads,V,dVdq,info)` (src/egrad_ch4h.f:74-79;
 * called from src/gradient.f90:178): natoms = 6 in Caracal's order H, C, H, H, H, H_b
 * (methane H = atoms 3,4,5,1; the abstracting H is atom 6), bohr -> Hartree. */
int cr_egrad_ch4h(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info);
/* Replaces `subroutine initialize_ch4h()` (src/egrad_ch4h.f:33, called from
 * src/read_pes.f90:551).  The surface's constants are compiled in, so this
 * only exists for call-site compatibility and always returns CR_OK. */
int cr_initialize_ch4h(void);

/* Replaces `subroutine egrad_ch4oh(q,Natoms,Nbeads,V,dVdq,info)` (src/egrad_ch4oh.f:69-124;
 * called from src/gradient.f90:180): natoms = 7 in Caracal's order H, C, H, H, H, O, H(O)
 * (methane H = atoms 3,4,5,1; O abstracts), bohr -> Hartree. */
int cr_egrad_ch4oh(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info);
/* egrad_oh3 (src/egrad_oh3.f:33-189): atoms O, H, H, H; natoms must be 4. */
int cr_egrad_oh3(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info);
/* Replaces `subroutine initialize_ch4oh()` (src/egrad_ch4oh.f:33, called from
 * src/read_pes.f90:591); constants are compiled in, always CR_OK. */
int cr_initialize_ch4oh(void);

/* Replaces `subroutine egrad_geh4oh(q,Natoms,Nbeads,V,dVdq,info)` (src/egrad_geh4oh.f:33-67;
 * called from src/gradient.f90:192-193 with Nbeads = 1): natoms = 7 in Caracal's order
 * H, Ge, H, H, H, O, H(O) (the CH4 + OH roles with Ge for C).  The reference routine reads
 * bead 1 only; this one evaluates every bead. */
int cr_egrad_geh4oh(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info);
/* Replaces `subroutine initialize_geh4oh()` (src/egrad_geh4oh.f:1823, called from
 * src/read_pes.f90:629); constants are compiled in, always CR_OK. */
int cr_initialize_geh4oh(void);

/* Replaces `subroutine egrad_brh2(q,Natoms,Nbeads,V,dVdq,info)` (src/egrad_brh2.f:33-78;
 * called from src/gradient.f90:182-183): natoms = 3 in Caracal's order H, Br, H. */
int cr_egrad_brh2(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info);
/* Replaces `subroutine initialize_brh2()` (src/egrad_brh2.f:80-130, called from
 * src/read_pes.f90:452); the set-up is compiled in, always CR_OK. */
int cr_initialize_brh2(void);

/* Any built PES (CR_PES_*) on device-resident arrays q(3,natoms,npts). */
int cr_egrad_device(int pes, const double* d_q, int npts, double* d_V, double* d_dVdq, int precision,
                    void* stream);

/* ---- QMDFF force field ------------------------------------------------------
 * Replaces the QMDFF branch of `gradient` (src/gradient.f90:342-358):
 * `ff_eg(n,at,xyz,e,g)` (src/ff_eg.f90:41) + `ff_nonb(n,at,xyz,q,r0ab,zab,
 * r0094,sr42,c66ab,enb,g)` (src/ff_nonb.f90:34) + `ff_hb(n,at,xyz,eh,g)`
 * (src/ff_hb.f90:36) + E_zero, one molecule, not periodic.  The arrays are those of module
 * qmdff (src/qmdff.f90:52-57, 1-based atom indices, Fortran column-major) and
 * the ff_nonb arguments; they are copied to the device at creation. */
typedef struct cr_qmdff_def {
  int natoms;
  const int* at;          /* at(natoms): element numbers 1..94 */
  const double* q;        /* q(natoms): charges */
  const double* rad;      /* rad(94): covalent radius per element, bohr (module qmdff) */
  int nbond, nangl, ntors, nnci;
  const int* bond;        /* bond(2,nbond) */
  const double* vbond;    /* vbond(3,nbond): r0, k, a */
  const int* angl;        /* angl(3,nangl): centre, i, k */
  const double* vangl;    /* vangl(2,nangl): theta0, k */
  const int* tors;        /* tors(6,ntors): i, j, k, l, nt, type (2 = inversion) */
  const double* vtors;    /* vtors(14,ntors): phi0, V, (rn, phase, Vn) x 4 */
  const int* nci;         /* nci(3,nnci): i, j, category 1..6 */
  const double* r0ab;     /* r0ab(94,94): repulsion exponent alpha */
  const double* zab;      /* zab(94,94) */
  const double* r0094;    /* r0094(94,94): BJ radius R0 */
  const double* sr42;     /* sr42(94,94) */
  const double* c66ab;    /* c66ab(natoms,natoms): pair C6 */
  double eps1[6], eps2[6];/* setnonb category scalings (src/setnonb.f90:164-190) */
  double coul_cut;        /* bohr: 50 (NVT) or 10 (NVE Zahn, src/dynamic.f90) */
  int zahn;               /* 1: Zahn Coulomb q q (erfc(a r)/r - par (r - cut)), no eps1 */
  double zahn_a, zahn_par;
  double e_zero;          /* E_zero1 shift */
  int nhb;                /* H/halogen bonds (src/ff_hb.f90; one molecule: the listed triples) */
  const int* hb;          /* hb(3,nhb): A, B, H (H bond if at(H) = 1, else halogen bond) */
  const double* vhb;      /* vhb(2,nhb): rdsolvff's hbpara * scalehb / scalexb values */
} cr_qmdff_def;
typedef struct cr_qmdff cr_qmdff;
int cr_qmdff_create(const cr_qmdff_def* def, cr_qmdff** out);
/* Periodic boundaries for the force field (PERIODIC x y z in Caracal's key
 * file; set_periodic, src/set_periodic.f90:67-113, and box_image,
 * src/box_image.f90:36-63): box edges and the Coulomb and dispersion
 * cutoffs in Angstrom (Caracal's defaults 50 and 10); a Coulomb cutoff below
 * 5 bohr becomes half the shortest edge minus 0.1 bohr, the Zahn form (as
 * the force field was created) fixes it at 10 A with its parameters, and no
 * Coulomb cutoff exceeds half the shortest edge.  Dispersion and repulsion
 * then act within the dispersion cutoff only.  Every distance vector of
 * every term is minimum-image (Caracal images the bond, angle, damping,
 * pair and H-bond vectors, and takes dihedrals from raw coordinates, which
 * agree for molecules not split across the box).  cuts (may be NULL)
 * receives coul_cut, vdw_cut, zahn_a, zahn_par as set (bohr).
 * box_ang NULL switches periodicity off.  Call it before an engine using
 * the force field is created. */
int cr_qmdff_set_periodic(cr_qmdff* ff, const double* box_ang, double coul_cut_ang, double vdw_cut_ang,
                          double* cuts);
/* Element tables for reading a .qmdff file: the (94,94) arrays ff_nonb takes
 * and, per element pair, the C6 that gives c6xy(i, j) = c6ab(at(i), at(j)). */
typedef struct cr_qmdff_tables {
  const double* rad;    /* rad(94), bohr */
  const double* r0ab;   /* (94,94) */
  const double* zab;
  const double* r0094;
  const double* sr42;
  const double* c6ab;   /* (94,94) */
} cr_qmdff_tables;
/* rdsolvff (src/rdsolvff.f90:34-202) from a file: the force field with E_zero
 * e_zero, the Zahn Coulomb switch and cutoff; H/halogen-bond strengths as
 * rdsolvff derives them from the charges (src/rdsolvff.f90:142-152). */
int cr_qmdff_load(const char* path, const cr_qmdff_tables* tab, double e_zero, int zahn, double coul_cut,
                  cr_qmdff** out);
/* Grimme's D3 reference data as Caracal's module qmdff holds it after
 * copyc6 (src/copyc6.f90, src/qmdff.f90:91): c6ab(94,94,5,5,3) column-major
 * (C6, CN of the first element, CN of the second per reference pair; -1
 * where none), maxci(94) reference CNs per element, rcov(94) the D3
 * covalent radii of the coordination number (src/setnonb.f90:80-101). */
typedef struct cr_d3_reference {
  const double* c6ab;
  const int* maxci;
  const double* rcov;
} cr_d3_reference;
/* rdsolvff + prepare (src/rdsolvff.f90:34-202, src/prepare.f90:100-129):
 * reads the .qmdff file, computes the coordination numbers of its reference
 * geometry (ncoord_qmdff, src/ncoord_qmdff.f90:36-76) and the CN-interpolated
 * pair C6 (getc6, src/getc6.f90:35-83), and builds the device force field
 * with the element tables of tab (its c6ab is not used; may be NULL). */
int cr_qmdff_load_d3(const char* path, const cr_qmdff_tables* tab, const cr_d3_reference* d3, double e_zero,
                     int zahn, double coul_cut, cr_qmdff** out);
/* natoms and the term counts (bonds, angles, torsions, H bonds, NCI pairs) of
 * a .qmdff file; host only. */
int cr_qmdff_file_counts(const char* path, int* natoms, int* counts);
int cr_qmdff_destroy(cr_qmdff* ff);
/* Host arrays xyz(3,natoms,nbeads) -> e(nbeads) (with E_zero), g(3,natoms,nbeads). */
int cr_qmdff_egrad(cr_qmdff* ff, const double* xyz, int nbeads, double* e, double* g, int precision);
/* cr_qmdff_egrad with each bead's virial trace vir[b] as the reference's
 * ff_eg / ff_nonb / ff_hb accumulate vir_ten with calc_vir (NpT; the
 * pressure takes its diagonal, src/verlet.f90:1123-1131): the terms'
 * formulas of src/ff_eg.f90:138-150, 270-281, 420-440, 583-603,
 * src/ff_nonb.f90:180-190, 318-328, 405-415, 495-505, src/eabhag.f90:203-216,
 * src/eabxag.f90:140-153 (the torsion, inversion and halogen-bond forms are
 * not the sum of (r - r_ref).g over the term's atoms; reproduced).  box: the
 * edges of bead b at box[3 b .. 3 b + 2] (bohr), NULL for the force field's;
 * the force field must be periodic (cr_qmdff_set_periodic). */
int cr_qmdff_egrad_virial(cr_qmdff* ff, const double* xyz, int nbeads, const double* box, double* e, double* g,
                          double* vir, int precision);
/* The three pieces of Caracal's QMDFF call site (src/gradient.f90:341-358),
 * for a caller that redirects them one by one; same arrays as
 * cr_qmdff_egrad, E_zero in none of them.
 *   cr_qmdff_eg:   bonds, angles, torsions and inversions; OVERWRITES e, g
 *                  (ff_eg, src/ff_eg.f90:41-72).
 *   cr_qmdff_nonb: dispersion, repulsion and Coulomb over the NCI pairs;
 *                  ADDS to e, g (ff_nonb, src/ff_nonb.f90:34, 886).
 *   cr_qmdff_hb:   hydrogen and halogen bonds; ADDS to e, g (ff_hb,
 *                  src/ff_hb.f90:36-280).
 * eg + nonb + hb + E_zero equals cr_qmdff_egrad to rounding. */
int cr_qmdff_eg(cr_qmdff* ff, const double* xyz, int nbeads, double* e, double* g, int precision);
int cr_qmdff_nonb(cr_qmdff* ff, const double* xyz, int nbeads, double* e, double* g, int precision);
int cr_qmdff_hb(cr_qmdff* ff, const double* xyz, int nbeads, double* e, double* g, int precision);

/* Derivatives for parameter fitting and adjoints (plain FP64 form; force
 * fields without H/halogen bonds, else CR_ERR_UNSUPPORTED).  No reference
 * counterpart: Caracal fits EVB couplings by finite differences (fdjac2) and
 * has no QMDFF force-constant gradients.
 * Linear parameters, in this order (count from cr_qmdff_nparams): bond force
 * constants k (vbond(2,:) of src/qmdff.f90), angle force constants (vangl(2,:)),
 * torsion barriers V (vtors(2,:)), NCI pair Coulomb products qq (eps1 q_i q_j,
 * or q_i q_j in the Zahn form).  Every term of ff_eg/ff_nonb is linear in its
 * parameter. */
int cr_qmdff_nparams(const cr_qmdff* ff, int* nlin);
/* hw[b] = Hessian of E at xyz[b] times w[b] (forward-mode dual numbers on the
 * term formulas); e, g (may be NULL) as cr_qmdff_egrad. */
int cr_qmdff_hvp(cr_qmdff* ff, const double* xyz, const double* w, int nbeads, double* e, double* g, double* hw);
/* grad[t] = d/dtheta_t sum_b v[b] . grad E(xyz[b]): the parameter gradient of
 * a force-matching loss with v = -dL/dF. */
int cr_qmdff_param_vjp(cr_qmdff* ff, const double* xyz, const double* v, int nbeads, double* grad);
/* Same on device-resident arrays; stream may be 0. */
int cr_qmdff_egrad_device(cr_qmdff* ff, const double* d_xyz, int nbeads, double* d_e, double* d_g,
                          int precision, void* stream);
/* Term batches of the mixed form's warp schedule (batches[5]: bonds, angles,
 * torsions, NCI pairs, H/halogen bonds) and the colours they need
 * (diagnostics; the plain form uses full 32-term batches). */
int cr_qmdff_schedule_info(const cr_qmdff* ff, int* batches, int* colors);
/* No counterpart in Caracal.  The force kernel comes in three occupancy
 * variants per form; the first launch of >= 2048 beads outside a stream
 * capture times each once and keeps the fastest.  variant = -1 before that;
 * ms[3] = the measured times. */
int cr_qmdff_tuning(const cr_qmdff* ff, int precision, int* variant, float* ms);

/* ---- dE-EVB of two QMDFFs ---------------------------------------------------
 * Replaces the two-QMDFF branch of `gradient` (src/gradient.f90:361-386 and
 * 1228-1304, EVB_QMDFF with a dE coupling, keyword DE_EVB): each force
 * field's energy includes its E_zero (cr_qmdff_def.e_zero = E_zero1 / E_zero2),
 * dE = E1 - E2, V12 = the coupling of the basis, E = (E1 + E2 -
 * sqrt(dE^2 + 4 V12^2)) / 2 and its analytic gradient as Caracal writes it. */
#define CR_EVB_CONST 0  /* V = a */
#define CR_EVB_1G 1     /* V = a exp(-b dE^2) */
#define CR_EVB_2G 2     /* + c exp(-d (dE+m)^2) */
#define CR_EVB_3G 3     /* + e exp(-f (dE+n)^2) */
#define CR_EVB_SP 4     /* a exp(-b dE^2) + c dE exp(-d dE^2) */
#define CR_EVB_SD 5     /* a exp(-b dE^2) + c dE^2 exp(-d dE^2) */
#define CR_EVB_SD2 6    /* + e dE^2 exp(-f dE^2) */
#define CR_EVB_SP2D 7   /* a exp(-b dE^2) + c dE exp(-d dE^2) + e dE exp(-f dE^2) + g dE^2 exp(-h dE^2) */
typedef struct cr_evb_def {
  int basis;                               /* CR_EVB_* (Caracal's off_basis) */
  double a, b, c, d, e, f, g, h, m, n;     /* offa..offh, offm, offn */
} cr_evb_def;
typedef struct cr_evb cr_evb;
/* Both force fields must describe the same atoms and outlive the EVB object. */
int cr_evb_create(cr_qmdff* ff1, cr_qmdff* ff2, const cr_evb_def* def, cr_evb** out);
int cr_evb_destroy(cr_evb* evb);
/* Host arrays xyz(3,natoms,nbeads) -> e(nbeads), g(3,natoms,nbeads). */
int cr_evb_egrad(cr_evb* evb, const double* xyz, int nbeads, double* e, double* g, int precision);

/* dE-EVB coupling fit (Caracal's EVB optimisation, src/optimize_de.f90 with
 * lm_de_func src/lm_de_func.f90:35-181): for m reference points with QMDFF
 * energies e1, e2 (E_zero included) and reference energies eref,
 * fvec[i] = (eref_i - E_EVB,i(x))^2 with dE = |e1 - e2|, and, if fjac is not
 * NULL, MINPACK's forward-difference Jacobian fdjac2 (src/lm_good.f:795-840,
 * epsfcn = 0) as fjac[j * m + i] = d fvec_i / d x_j.  Parameters x per basis:
 * 1g a b | 2g a b c d m | 3g a b c d e f m n | sp, sd a b c d | sd2 a b c d e f |
 * sp2d a .. h | sp2d3 a .. l. */
#define CR_FIT_1G 1
#define CR_FIT_2G 2
#define CR_FIT_3G 3
#define CR_FIT_SP 4
#define CR_FIT_SD 5
#define CR_FIT_SD2 6
#define CR_FIT_SP2D 7
#define CR_FIT_SP2D3 8
int cr_evb_fit(int basis, const double* x, int npar, int m, const double* e1, const double* e2, const double* eref,
               double* fvec, double* fjac);
/* grad[j] = d/dx_j sum_i fvec_i: the analytic gradient of the fit loss (dual
 * numbers), against which the fdjac2 columns summed over the points are the
 * reference's finite-difference counterpart. */
int cr_evb_fit_grad(int basis, const double* x, int npar, int m, const double* e1, const double* e2,
                    const double* eref, double* grad);
/* Parameter gradient of sum_b v[b] . grad E_EVB(xyz[b]) (a force-matching loss
 * with v = -dL/dF), plain FP64: grad_coupling[10] over the coupling
 * parameters a..h, m, n of cr_evb_def, and, if grad_ff1 is not NULL, over the
 * first force field's linear parameters (order of cr_qmdff_param_vjp). */
int cr_evb_param_vjp(cr_evb* evb, const double* xyz, const double* v, int nbeads, double* grad_coupling,
                     double* grad_ff1);

/* ---- RPMD engine -----------------------------------------------------------
 * Replaces the stepping loop of `dynamic` (src/dynamic.f90:1569-1579) around
 * `verlet` (src/verlet.f90:65) and the initialisation of `mdinit`
 * (src/mdinit.f90:40-173), batched over ntraj independent trajectories. */
int cr_engine_create(const cr_config* cfg, cr_engine** out);
/* Engine on a QMDFF (cfg->pes = CR_PES_QMDFF, cfg->natoms = the force
 * field's natoms, cfg->mass natoms masses).  The force field must outlive the
 * engine.  Steps run as a CUDA graph of kernels (kick + free ring polymer,
 * forces, kick + thermostat, transrot) instead of one persistent launch. */
int cr_engine_create_qmdff(const cr_config* cfg, cr_qmdff* ff, cr_engine** out);
/* Engine on a dE-EVB of two QMDFFs (cfg->pes = CR_PES_EVB); the EVB object
 * and its force fields must outlive the engine. */
int cr_engine_create_evb(const cr_config* cfg, cr_evb* evb, cr_engine** out);
/* Engine on a water box (cfg->pes = CR_PES_WATER, cfg->natoms = 3 nwater);
 * the box must outlive the engine.  Steps run through the graph path. */
int cr_engine_create_water(const cr_config* cfg, cr_water* w, cr_engine** out);
int cr_engine_destroy(cr_engine* e);

/* Initial positions: every bead of every trajectory = q0(3,natoms) plus
 * sigma * N(0,1) per coordinate (sigma in bohr; 0 gives Caracal's identical
 * beads, src/dynamic.f90:1307-1314). */
int cr_engine_init_positions(cr_engine* e, const double* q0, double sigma);
/* mdinit momenta: Andersen draw (NVT, src/mdinit.f90:118-121) or zeros
 * (NVE, src/mdinit.f90:125). */
int cr_engine_init_momenta(cr_engine* e, int zero);
/* mdinit forces (src/mdinit.f90:80-83) of the current positions. */
int cr_engine_compute_forces(cr_engine* e);

/* Host <-> engine state, arrays (3, natoms, nbeads, ntraj).  f (dV/dq of the
 * current positions) may be NULL in set_state; it is then recomputed. */
int cr_engine_set_state(cr_engine* e, const double* q, const double* p, const double* f);
int cr_engine_get_state(cr_engine* e, double* q, double* p, double* f, double* epot, int* status);

/* Advances every trajectory by nsteps steps in one persistent launch; the
 * step counter continues from previous runs.  Returns CR_ERR_TRAJECTORY if a
 * trajectory reported a status bit (state is still returned). */
int cr_engine_run(cr_engine* e, int nsteps);
/* cr_engine_run with Caracal's trajectory dumps (src/verlet.f90:780-800,
 * every iwrite steps): after each step whose index is a multiple of `every`
 * the state is copied to the caller's q, p (3 x natoms x nbeads x ntraj) and
 * epot (ntraj) and dump(user, istep, q, p, epot) is called; a nonzero return
 * stops the run with CR_ERR_ARG. */
typedef int (*cr_dump_fn)(void* user, int istep, const double* q, const double* p, const double* epot);
int cr_engine_run_dump(cr_engine* e, int nsteps, int every, cr_dump_fn dump, void* user, double* q, double* p,
                       double* epot);
/* The same dumps without holding up the stepping (replaces the synchronous
 * dumps of src/verlet.f90:780-800): at each dump step the state is copied to
 * one of two device snapshot slots on the engine's stream and from there to
 * page-locked host memory on a second stream, while the next steps run.
 * dump() receives a snapshot (pointers into the library's page-locked
 * buffers, valid during the call) one dump late, so writing frames to disk
 * overlaps the dynamics; the last snapshot is delivered before the call
 * returns.  A trajectory whose status word is set by a dump step ends the
 * run with CR_ERR_TRAJECTORY before that frame is handed over.  The slots
 * (2 x (2 T P 3N + T) doubles + 2 T ints, device and host) are allocated on
 * the first call and kept until cr_engine_destroy. */
int cr_engine_run_dump_async(cr_engine* e, int nsteps, int every, cr_dump_fn dump, void* user);

/* One `verlet` step through host buffers, as a Fortran caller holding
 * q_i, p_i, derivs would use it: copy in, one step, copy out (epot may be NULL). */
int cr_engine_step_host(cr_engine* e, double* q, double* p, double* f, double* epot);

/* ---- recrossing children (calc_rate part 4) --------------------------------
 * Replaces the child loop of `recross` (src/recross.f90:540-614): children in
 * pairs with momenta +p and -p (Andersen draw at the engine's temperature),
 * started from one parent ring polymer, run NVE without thermostat or
 * transrot (verlet with constrain = 2); after every step the BIMOLEC reaction
 * coordinate of the centroid (calc_xi mode 2, src/calc_xi.f90) decides the
 * side.  kappa(t) = num[t] / denom (src/recross.f90:637). */
typedef struct cr_recross {
  int nreac1, reac1[8];        /* MECHA reactant1 atoms, 1-based */
  int nreac2, reac2[8];        /* MECHA reactant2 atoms, 1-based */
  int bond_form[2];            /* MECHA bond_form atoms, 1-based */
  int bond_break[2];           /* MECHA bond_break atoms, 1-based */
  double form_ref, break_ref;  /* bond lengths at the TS, bohr (src/bonds_ref.f90) */
  double r_inf;                /* DIST_INF, bohr */
  double xi_ideal;             /* xi of the dividing surface (PMF maximum) */
} cr_recross;
/* Enables the flux bookkeeping for runs of at most max_steps steps in total
 * after the next cr_engine_init_children.  The engine must be created with
 * thermostat CR_THERMO_NONE and transrot 0 to reproduce child steps. */
int cr_engine_set_recross(cr_engine* e, const cr_recross* rc, int max_steps);
/* q_parent(3,natoms,nbeads): every child starts there; pairs (2i, 2i+1) get
 * +p/-p from the Gaussian stream keyed by traj0 + 2i; forces and the flux
 * weights vs/fs are computed. */
int cr_engine_init_children(cr_engine* e, const double* q_parent);
/* num[nsteps] and denom summed over the engine's children (deterministic
 * order); weights (may be NULL) gets vs/fs per child. */
int cr_engine_kappa(cr_engine* e, double* num, double* denom, double* weights, int* nsteps);

/* Constrained parent trajectories (calc_rate part 3, src/recross.f90:240-290:
 * verlet with constrain = 1): after each free ring-polymer step SHAKE moves
 * the centroid onto xi = 0 of the BIMOLEC coordinate rc (src/constrain_q.f90),
 * after the second half kick RATTLE removes the momentum along dxi
 * (src/constrain_p.f90); no transrot.  Call once after the initial state is
 * set (dxi starts at the current centroid); the engine then steps through its
 * kernel-graph path.  Analytic surfaces only. */
int cr_engine_set_parent(cr_engine* e, const cr_recross* rc);

/* Device time of the last cr_engine_run / step kernel (CUDA events on the
 * engine's stream), launches issued by it, and the launch shape chosen. */
int cr_engine_last_kernel_ms(const cr_engine* e, float* ms);
int cr_engine_launch_info(const cr_engine* e, int* grid, int* block, int* smem_bytes, int* launches);
/* Device pointers of the state arrays (owned by the engine). */
int cr_engine_device_state(cr_engine* e, double** q, double** p, double** f);
/* Page-locked host buffers for fast host<->device copies. */
int cr_host_alloc(void** ptr, unsigned long long bytes);
int cr_host_free(void* ptr);
/* Page-lock memory the caller already owns (cudaHostRegister), e.g. the
 * module arrays q_i, p_i, derivs of Caracal's Fortran host (src/evb_mod.f90:246),
 * so that cr_engine_step_host copies them at pinned-memory speed instead of
 * staging pageable memory; unregister before the memory is freed. */
int cr_host_register(void* ptr, unsigned long long bytes);
int cr_host_unregister(void* ptr);

/* ---- pipe calibration (no reference counterpart) ---------------------------
 * Device throughput (operations per second over the whole GPU) of one
 * operation class in FP64 (fp64 = 1) or FP32: used to weight counted
 * transcendentals and divisions in FMA-equivalents for the roofline. */
#define CR_CALIB_FMA 0
#define CR_CALIB_DIV 1
#define CR_CALIB_SQRT 2
#define CR_CALIB_EXP 3
#define CR_CALIB_LOG 4
#define CR_CALIB_POW 5
#define CR_CALIB_SIN 6
#define CR_CALIB_COS 7
#define CR_CALIB_ACOS 8
#define CR_CALIB_ERF 9
#define CR_CALIB_TANH 10
#define CR_CALIB_COSH 11
/* FP64 tensor-core MMA (mma.sync m8n8k4 f64, 256 multiply-adds per warp
 * instruction), reported in multiply-adds per second (fp64 must be 1): the
 * A/B of the bead transform as a dense contraction against DFMA code. */
#define CR_CALIB_DMMA 12
int cr_calibrate_op(int fp64, int op, int iters, double* ops_per_s);

/* ---- umbrella windows (calc_rate's umbrella sampling) ----------------------
 * Trajectory t samples the window centred at centers[t] with force constant
 * kforce[t] (Eh; Caracal scales its UMBR_BONDS input by the temperature,
 * src/calc_rate.f90:699): after the forces of every step, each bead's gradient
 * gets k (xi - xi_t) dxi and the gradient of -(1/beta) log fs at the centroid
 * (src/umbrella.f90:100-176, xi of calc_xi mode 1 on the MECHA definition rc).
 * Analytic surfaces, finite temperature.  With sampling on, the xi of every
 * step is summed (xsum, xsum2) and binned into nbins over [lo, hi): the
 * averages and variances of umbrella integration and the histograms of WHAM
 * (src/calc_rate.f90:1568-1700, 1936-2012). */
int cr_engine_set_umbrella(cr_engine* e, const cr_recross* rc, const double* centers, const double* kforce,
                           int nbins, double lo, double hi);
int cr_engine_umbrella_sampling(cr_engine* e, int on);
/* xsum[T], xsum2[T], hist[T][nbins] (each may be NULL); reset != 0 zeroes them */
int cr_engine_umbrella_stats(cr_engine* e, double* xsum, double* xsum2, double* hist, int reset);

/* Caracal's mdinit (src/mdinit.f90:40-173) as calc_rate calls it before
 * every window trajectory and every parent segment (src/calc_rate.f90:966,
 * 1536; src/recross.f90:251,462): forces of the current positions, plus the
 * umbrella bias of mode 0 where the engine has umbrella windows
 * (src/mdinit.f90:96-100; sampling must be off), then Andersen momenta (NVT,
 * src/mdinit.f90:118-121) or zeros (NVE, :125), the Nose-Hoover chain at
 * rest.  `draw` numbers the Gaussian stream of the momenta: draw 0 is the
 * stream of cr_engine_init_momenta, and a later call with a new draw gives
 * fresh momenta, as each of Caracal's mdinit calls does. */
int cr_engine_mdinit(cr_engine* e, unsigned draw);
/* ANDERSEN_STEP of an existing engine.  Caracal's recrossing sets it per
 * phase of the parent trajectory: int(sqrt(equi_steps)) for the
 * equilibration, int(sqrt(child_interval)) between child batches
 * (src/recross.f90:239-242, 456-458). */
int cr_engine_set_andersen_step(cr_engine* e, int andersen_step);

/* NpT with the Berendsen barostat (ENSEMBLE NPT, BAROSTAT BERENDSEN,
 * src/verlet.f90:1111-1151; constants of src/mdinit.f90:155-158) for an
 * engine on one periodic QMDFF: every trajectory keeps its own box, starting
 * from box_bohr[3 t .. 3 t + 2] (NULL: the force field's box).  Each step
 * sums the beads' virial traces (the terms' vir_ten as the reference forms
 * them), takes the pressure as -tr W / (3 V) (the reference's kinetic
 * stress tensor stays zero) and after the second half kick scales the box
 * and the coordinates by (1 + dt compress / taupres (p - p0))^(1/3),
 * p0 = pressure_atm / prescon.  A Nose-Hoover chain thermostat is not
 * applied under it (the reference calls neither nhc nor nhc_npt there).
 * CR_ERR_UNSUPPORTED for other force fields, dE-EVB, constrained parents and
 * umbrella windows. */
int cr_engine_set_npt(cr_engine* e, double pressure_atm, const double* box_bohr);
/* Each trajectory's box edges (bohr, T x 3), its last step's pressure and
 * the sum of its pressures since the last reset (a.u.; x prescon =
 * 290371576.61 for atm; Caracal prints that sum / iwrite as press_avg,
 * src/verlet.f90:1171-1210); any pointer may be NULL; reset_sum != 0 zeroes
 * the sums after reading. */
int cr_engine_get_npt(cr_engine* e, double* box_bohr, double* pressure_au, double* pressure_sum_au, int reset_sum);

/* Launch shape of the persistent step kernel (analytic surfaces; the graph
 * path of force fields has none and returns CR_ERR_UNSUPPORTED).  A
 * trajectory's beads sit on G = next_pow2(nbeads) threads, each served by
 * threads_per_bead (1, 2 or 4; 4 is built for H3 and OH + H2, 1 for CH4 + H
 * and CH4 + OH) threads that split the bead's atoms between them for the
 * integrator's per-coordinate work; threads_per_block (a multiple of
 * G x threads_per_bead, <= 256) sets how many trajectories share a block.
 * threads_per_block = 0 restores the built-in choice (one thread per bead,
 * 32 threads per block for a batch of at most 128 threads per SM, else 128).
 * No counterpart in the reference, which steps one trajectory at a time on
 * the host. */
int cr_engine_set_launch(cr_engine* e, int threads_per_block, int threads_per_bead);
int cr_engine_get_launch(cr_engine* e, int* threads_per_block, int* blocks, int* threads_per_bead);
/* Autotuner: times nsteps steps at each launch shape (threads per bead 1, 2,
 * 4 as built; G x threads_per_bead, 32, 64, 128, 256 threads per block, those
 * that fit), each from the same saved state, which is then put back (q, p,
 * f, epot, status, chain velocities, step counter); keeps the fastest and
 * returns it with its time per step.  The noise is a function of the step
 * index, so the trials leave no trace in the run. */
int cr_engine_autotune(cr_engine* e, int nsteps, int* threads_per_block, int* threads_per_bead,
                       float* ms_per_step);

/* ---- batches of trajectory classes -----------------------------------------
 * One graph launch per chunk of steps advances several engines (classes with
 * different surfaces, atom and bead counts, precisions) side by side: Caracal
 * farms such runs over MPI ranks (src/dynamic.f90:1569-1579 per rank); here
 * they share one GPU.  Each engine keeps its own state and step counter;
 * cr_batch_run(b, n) is cr_engine_run(e, n) for every engine of the batch
 * (the same results) with the classes overlapped on the device. */
typedef struct cr_batch cr_batch;
int cr_batch_create(cr_engine* const* engines, int nengines, int chunk_steps, cr_batch** out);
int cr_batch_run(cr_batch* b, int nsteps);
/* kernels launched by the last cr_batch_run, kernels per chunk graph, its
 * device time in ms */
int cr_batch_info(const cr_batch* b, long long* launches, int* graph_nodes, float* ms);
/* Timeline of the last graph launch of cr_batch_run: per engine, when its
 * branch began and ended, in ms after the launch began (events recorded
 * inside the graph).  Branches whose intervals overlap ran concurrently. */
int cr_batch_timeline(const cr_batch* b, float* begin_ms, float* end_ms);
int cr_batch_destroy(cr_batch* b);

/* ---- adjoint of the step (parameter fitting through trajectories) --------
 * No reference counterpart.  For a QMDFF engine in the plain FP64 form with
 * NVE steps (thermostat CR_THERMO_NONE, transrot 0): cr_adjoint_forward runs
 * nsteps steps from the engine's current state, keeping (q, p, dV/dq) every
 * `every` steps; cr_adjoint_backward takes dL/dq and dL/dp of a loss of the
 * final state (host arrays shaped like the state) and returns dL/dtheta over
 * the force field's linear parameters (order of cr_qmdff_param_vjp) and,
 * if not NULL, dL/dq and dL/dp of the initial state.  Each segment's
 * positions are recomputed from its checkpoint; the engine ends in its state
 * after the forward run. */
typedef struct cr_adjoint cr_adjoint;
int cr_adjoint_create(cr_engine* e, int nsteps, int every, cr_adjoint** out);
int cr_adjoint_forward(cr_adjoint* a);
int cr_adjoint_backward(cr_adjoint* a, const double* dl_dq, const double* dl_dp, double* grad, double* dl_dq0,
                        double* dl_dp0);
int cr_adjoint_destroy(cr_adjoint* a);

#ifdef __cplusplus
}
#endif
#endif /* CARACAL_GB300_H */
