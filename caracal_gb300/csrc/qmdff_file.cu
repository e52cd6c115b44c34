// Caracal's .qmdff file (src/rdsolvff.f90:34-202; written by qmdffgen,
// src/main_gen.f90:825-847) read on the host into a cr_qmdff: the C-ABI
// counterpart of `rdsolvff` + `prepare` for callers that hold a file name,
// not module arrays.  Each list-directed READ starts on a new line and takes
// values over as many lines as it needs; the rest of its last line is
// skipped.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "host_util.h"
#include "qmdff_host.h"

namespace {

struct Records {
  std::vector<std::string> lines;
  size_t pos = 0;
  // n values of one list-directed READ (Fortran D exponents accepted)
  bool read(size_t n, std::vector<std::string>& out) {
    out.clear();
    while (out.size() < n) {
      if (pos >= lines.size()) return false;
      std::string ln = lines[pos++];
      for (char& c : ln)
        if (c == 'D' || c == 'd') c = 'E';
      std::istringstream is(ln);
      std::string tok;
      while (is >> tok) out.push_back(tok);
    }
    out.resize(n);
    return true;
  }
};

struct FileFF {
  int n = 0, nbond = 0, nangl = 0, ntors = 0, nhb = 0, nnci = 0;
  std::vector<int> at, bond, angl, tors, hb, nci;
  std::vector<double> q, xyz, vbond, vangl, vtors;  // xyz(3, n): reference geometry, bohr
};

int parse(const char* path, FileFF& f) {
  std::ifstream in(path);
  if (!in) return cr_set_error(CR_ERR_ARG, std::string("cannot open ") + path);
  Records r;
  std::string ln;
  while (std::getline(in, ln)) r.lines.push_back(ln);
  std::vector<std::string> v;
  auto toi = [](const std::string& s) { return (int)std::lround(std::atof(s.c_str())); };
  auto tod = [](const std::string& s) { return std::atof(s.c_str()); };
  if (!r.read(1, v)) return cr_set_error(CR_ERR_ARG, "empty .qmdff file");
  f.n = toi(v[0]);
  if (f.n < 1 || f.n > 1024) return cr_set_error(CR_ERR_ARG, "atom count of the .qmdff file out of 1..1024");
  r.pos = 2;  // the second line holds the method name
  for (int i = 0; i < f.n; ++i) {
    if (!r.read(6, v)) return cr_set_error(CR_ERR_ARG, "truncated atom block");
    f.at.push_back(toi(v[0]));
    for (int k = 1; k < 4; ++k) f.xyz.push_back(tod(v[(size_t)k]));
    f.q.push_back(tod(v[4]));
  }
  if (!r.read(5, v)) return cr_set_error(CR_ERR_ARG, "missing term counts");
  f.nbond = toi(v[0]);
  f.nangl = toi(v[1]);
  f.ntors = toi(v[2]);
  f.nhb = toi(v[3]);
  f.nnci = toi(v[4]);
  if (f.nbond < 0 || f.nangl < 0 || f.ntors < 0 || f.nhb < 0 || f.nnci < 0)
    return cr_set_error(CR_ERR_ARG, "negative term count");
  for (int m = 0; m < f.nbond; ++m) {
    if (!r.read(5, v)) return cr_set_error(CR_ERR_ARG, "truncated bond block");
    f.bond.push_back(toi(v[0]));
    f.bond.push_back(toi(v[1]));
    for (int k = 2; k < 5; ++k) f.vbond.push_back(tod(v[k]));
  }
  for (int m = 0; m < f.nangl; ++m) {
    if (!r.read(5, v)) return cr_set_error(CR_ERR_ARG, "truncated angle block");
    for (int k = 0; k < 3; ++k) f.angl.push_back(toi(v[k]));
    f.vangl.push_back(tod(v[3]));
    f.vangl.push_back(tod(v[4]));
  }
  const double pi = 3.1415926535897932384626433832795029;
  for (int m = 0; m < f.ntors; ++m) {
    // i j k l nt type phi0 V (rn phase/pi Vn) x nt on one record
    if (r.pos >= r.lines.size()) return cr_set_error(CR_ERR_ARG, "truncated torsion block");
    std::string line = r.lines[r.pos++];
    for (char& c : line)
      if (c == 'D' || c == 'd') c = 'E';
    std::istringstream is(line);
    std::vector<std::string> t;
    std::string tok;
    while (is >> tok) t.push_back(tok);
    if (t.size() < 8) return cr_set_error(CR_ERR_ARG, "short torsion record");
    const int nt = toi(t[4]);
    if (nt < 0 || nt > 4 || t.size() < (size_t)(8 + 3 * nt)) return cr_set_error(CR_ERR_ARG, "bad torsion record");
    for (int k = 0; k < 6; ++k) f.tors.push_back(toi(t[(size_t)k]));
    std::vector<double> w(14, 0.0);
    w[0] = tod(t[6]);
    w[1] = tod(t[7]);
    for (int j = 0; j < nt; ++j) {
      w[(size_t)2 + 3 * j] = tod(t[(size_t)8 + 3 * j]);
      w[(size_t)3 + 3 * j] = tod(t[(size_t)9 + 3 * j]) * pi;
      w[(size_t)4 + 3 * j] = tod(t[(size_t)10 + 3 * j]);
    }
    f.vtors.insert(f.vtors.end(), w.begin(), w.end());
  }
  if (f.nhb) {
    if (!r.read((size_t)3 * f.nhb, v)) return cr_set_error(CR_ERR_ARG, "truncated H-bond block");
    for (auto& s : v) f.hb.push_back(toi(s));
  }
  if (f.nnci) {
    if (!r.read((size_t)3 * f.nnci, v)) return cr_set_error(CR_ERR_ARG, "truncated NCI block");
    for (auto& s : v) f.nci.push_back(toi(s));
  }
  return CR_OK;
}

// rdsolvff's H/halogen-bond strengths (src/rdsolvff.f90:142-152) with the
// scalings of setnonb (src/setnonb.f90:123-137, REAL(4) literals).
double scale_hb(int z) {
  switch (z) {
    case 7: return (double)0.8f;
    case 8: return (double)0.3f;
    case 9: return (double)0.1f;
    case 15: case 16: case 17: case 34: case 35: return (double)2.0f;
    default: return 0.0;
  }
}
double scale_xb(int z) {
  switch (z) {
    case 17: return (double)0.30f;
    case 35: return (double)0.60f;
    case 53: return (double)0.80f;
    case 85: return 1.0;
    default: return 0.0;
  }
}
double hbpara(double a, double b, double q) { return std::exp(-a * q) / (std::exp(-a * q) + b); }

// Coordination numbers of the reference geometry (src/ncoord_qmdff.f90:36-76):
// cn_i = sum_j 1 / (1 + exp(-16 ((rcov_i + rcov_j) / r_ij - 1))), pairs with
// r^2 > cn_thr bohr^2 skipped.
void ncoord(const FileFF& f, const double* rcov, double cn_thr, std::vector<double>& cn) {
  const int n = f.n;
  cn.assign((size_t)n, 0.0);
  for (int i = 0; i < n; ++i) {
    double xn = 0.0;
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      const double dx = f.xyz[3 * (size_t)j] - f.xyz[3 * (size_t)i];
      const double dy = f.xyz[3 * (size_t)j + 1] - f.xyz[3 * (size_t)i + 1];
      const double dz = f.xyz[3 * (size_t)j + 2] - f.xyz[3 * (size_t)i + 2];
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 > cn_thr) continue;
      const double r = std::sqrt(r2);
      const double rr = (rcov[f.at[(size_t)i] - 1] + rcov[f.at[(size_t)j] - 1]) / r;
      xn = xn + 1.0 / (1.0 + std::exp(-16.0 * (rr - 1.0)));
    }
    cn[(size_t)i] = xn;
  }
}

// CN-interpolated pair C6 (src/getc6.f90:35-83) from the D3 reference table
// c6ab(94,94,5,5,3) (column-major, as copyc6 leaves module qmdff).
double getc6(const cr_d3_reference* d3, int iat, int jat, double nci, double ncj) {
  auto at5 = [&](int i, int j, int a, int b, int m) {
    return d3->c6ab[(size_t)(i - 1) + 94 * ((size_t)(j - 1) + 94 * ((size_t)a + 5 * ((size_t)b + 5 * (size_t)m)))];
  };
  double c6mem = -1e99, rsum = 0.0, csum = 0.0, r_save = 10000.0;
  for (int a = 0; a < d3->maxci[iat - 1]; ++a)
    for (int b = 0; b < d3->maxci[jat - 1]; ++b) {
      const double c6 = at5(iat, jat, a, b, 0);
      if (c6 > 0) {
        const double cn1 = at5(iat, jat, a, b, 1), cn2 = at5(iat, jat, a, b, 2);
        const double r = (cn1 - nci) * (cn1 - nci) + (cn2 - ncj) * (cn2 - ncj);
        if (r < r_save) {
          r_save = r;
          c6mem = c6;
        }
        const double tmp1 = std::exp(-4.0 * r);
        rsum = rsum + tmp1;
        csum = csum + tmp1 * c6;
      }
    }
  return rsum > 1e-99 ? csum / rsum : c6mem;
}

// Common tail of the loaders: H-bond strengths, eps scalings, the device force field.
int build_from_file(const FileFF& f, const cr_qmdff_tables* tab, const std::vector<double>& c6, double e_zero,
                    int zahn, double coul_cut, cr_qmdff** out);

}  // namespace

extern "C" {

int cr_qmdff_file_counts(const char* path, int* natoms, int* counts) {
  if (!path || !natoms || !counts) return cr_set_error(CR_ERR_ARG, "NULL argument");
  FileFF f;
  int rc = parse(path, f);
  if (rc) return rc;
  *natoms = f.n;
  counts[0] = f.nbond;
  counts[1] = f.nangl;
  counts[2] = f.ntors;
  counts[3] = f.nhb;
  counts[4] = f.nnci;
  return CR_OK;
}

int cr_qmdff_load(const char* path, const cr_qmdff_tables* tab, double e_zero, int zahn, double coul_cut,
                  cr_qmdff** out) {
  if (!path || !tab || !out || !tab->rad || !tab->r0ab || !tab->zab || !tab->r0094 || !tab->sr42 || !tab->c6ab)
    return cr_set_error(CR_ERR_ARG, "NULL argument");
  *out = nullptr;
  FileFF f;
  int rc = parse(path, f);
  if (rc) return rc;
  for (int z : f.at)
    if (z < 1 || z > 94) return cr_set_error(CR_ERR_ARG, "element number out of 1..94");
  const int n = f.n;
  std::vector<double> c6((size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) c6[(size_t)i + (size_t)n * j] = tab->c6ab[(size_t)(f.at[i] - 1) + 94 * (size_t)(f.at[j] - 1)];
  return build_from_file(f, tab, c6, e_zero, zahn, coul_cut, out);
}

int cr_qmdff_load_d3(const char* path, const cr_qmdff_tables* tab, const cr_d3_reference* d3, double e_zero,
                     int zahn, double coul_cut, cr_qmdff** out) {
  if (!path || !tab || !d3 || !out || !tab->rad || !tab->r0ab || !tab->zab || !tab->r0094 || !tab->sr42 ||
      !d3->c6ab || !d3->maxci || !d3->rcov)
    return cr_set_error(CR_ERR_ARG, "NULL argument");
  *out = nullptr;
  for (int z = 0; z < 94; ++z)
    if (d3->maxci[z] < 0 || d3->maxci[z] > 5) return cr_set_error(CR_ERR_ARG, "maxci out of 0..5");
  FileFF f;
  int rc = parse(path, f);
  if (rc) return rc;
  for (int z : f.at)
    if (z < 1 || z > 94) return cr_set_error(CR_ERR_ARG, "element number out of 1..94");
  // prepare (src/prepare.f90:121-129): CN of the file's geometry, pair C6
  std::vector<double> cn;
  ncoord(f, d3->rcov, 5000.0, cn);
  const int n = f.n;
  std::vector<double> c6((size_t)n * n);
  for (int i1 = 0; i1 < n; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2) {
      const double v = getc6(d3, f.at[(size_t)i1], f.at[(size_t)i2], cn[(size_t)i1], cn[(size_t)i2]);
      c6[(size_t)i2 + (size_t)n * i1] = v;
      c6[(size_t)i1 + (size_t)n * i2] = v;
    }
  return build_from_file(f, tab, c6, e_zero, zahn, coul_cut, out);
}

}  // extern "C"

namespace {

int build_from_file(const FileFF& f, const cr_qmdff_tables* tab, const std::vector<double>& c6, double e_zero,
                    int zahn, double coul_cut, cr_qmdff** out) {
  const int n = f.n;
  std::vector<double> vhb((size_t)2 * f.nhb, 0.0);
  for (int k = 0; k < f.nhb; ++k) {
    const int a = f.hb[(size_t)3 * k] - 1, b = f.hb[(size_t)3 * k + 1] - 1, h = f.hb[(size_t)3 * k + 2] - 1;
    if (a < 0 || b < 0 || h < 0 || a >= n || b >= n || h >= n) return cr_set_error(CR_ERR_ARG, "H-bond atom out of range");
    if (f.at[(size_t)h] == 1) {
      vhb[(size_t)2 * k] = hbpara(10.0, 5.0, f.q[(size_t)a]) * scale_hb(f.at[(size_t)a]);
      vhb[(size_t)2 * k + 1] = hbpara(10.0, 5.0, f.q[(size_t)b]) * scale_hb(f.at[(size_t)b]);
    } else {
      vhb[(size_t)2 * k] = scale_xb(f.at[(size_t)h]) * hbpara(-6.5, 1.0, f.q[(size_t)h]);
    }
  }
  cr_qmdff_def d{};
  d.natoms = n;
  d.at = f.at.data();
  d.q = f.q.data();
  d.rad = tab->rad;
  d.nbond = f.nbond;
  d.nangl = f.nangl;
  d.ntors = f.ntors;
  d.nnci = f.nnci;
  d.bond = f.bond.data();
  d.vbond = f.vbond.data();
  d.angl = f.angl.data();
  d.vangl = f.vangl.data();
  d.tors = f.tors.data();
  d.vtors = f.vtors.data();
  d.nci = f.nci.data();
  d.r0ab = tab->r0ab;
  d.zab = tab->zab;
  d.r0094 = tab->r0094;
  d.sr42 = tab->sr42;
  d.c66ab = c6.data();
  // setnonb's category scalings (src/setnonb.f90:164-190); eps1(3) = 0.85 is a REAL(4) literal
  const double eps1[6] = {0.0, 0.0, (double)0.85f, 1.0, 1.0, 0.0};
  const double eps2[6] = {0.0, 0.0, 0.5, 0.5, 1.0, 1.0};
  for (int k = 0; k < 6; ++k) {
    d.eps1[k] = eps1[k];
    d.eps2[k] = eps2[k];
  }
  d.coul_cut = coul_cut;
  d.zahn = zahn;
  d.zahn_a = 0.0;
  d.zahn_par = 0.0;
  d.e_zero = e_zero;
  d.nhb = f.nhb;
  d.hb = f.hb.data();
  d.vhb = vhb.data();
  return cr_qmdff_create(&d, out);
}

}  // namespace
