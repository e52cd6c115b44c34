// ORACLE (test infrastructure only) -- QMDFF's D3 dispersion set-up, CPU restatement.
//
//   copyc6        src/copyc6.f90:35674-35744  reference table c6ab(94,94,5,5,3), maxci(94)
//                                              from the pars lines (C6, code_i, code_j, CN_i, CN_j),
//                                              alkali / alkaline-earth C6 from the rare gas
//   limit         src/limit.f90:34-60         element code above 100 -> CN-reference index
//   ncoord_qmdff  src/ncoord_qmdff.f90:36-76  coordination numbers, k1 = 16, r^2 cut 5000 bohr^2
//   getc6         src/getc6.f90:35-83         exp(-4 r)-weighted C6 over the reference pairs
//   prepare       src/prepare.f90:121-129     c6xy(i2, i1) = c6xy(i1, i2) for i2 <= i1
#pragma once
#include <cmath>
#include <vector>

namespace orc {

struct D3Ref {
  // c6ab(i, j, a, b, m): element i, j (0-based), CN index a, b, m = C6 / CN_i / CN_j
  std::vector<double> c6ab = std::vector<double>((size_t)94 * 94 * 5 * 5 * 3, -1.0);
  int maxci[94] = {0};
  double& at(int i, int j, int a, int b, int m) {
    return c6ab[(((((size_t)i * 94 + j) * 5 + a) * 5 + b) * 3) + m];
  }
};

inline void limit(int& iat, int& iadr) {
  iadr = 1;
  while (iat > 100) {
    iat -= 100;
    iadr += 1;
  }
}

inline void copyc6(const double* pars, int nlines, D3Ref& d) {
  for (int nn = 0; nn < nlines; ++nn) {
    const double* p = pars + (size_t)5 * nn;
    int iat = (int)p[1], jat = (int)p[2], iadr, jadr;
    limit(iat, iadr);
    limit(jat, jadr);
    if (iadr > d.maxci[iat - 1]) d.maxci[iat - 1] = iadr;
    if (jadr > d.maxci[jat - 1]) d.maxci[jat - 1] = jadr;
    d.at(iat - 1, jat - 1, iadr - 1, jadr - 1, 0) = p[0];
    d.at(iat - 1, jat - 1, iadr - 1, jadr - 1, 1) = p[3];
    d.at(iat - 1, jat - 1, iadr - 1, jadr - 1, 2) = p[4];
    d.at(jat - 1, iat - 1, jadr - 1, iadr - 1, 0) = p[0];
    d.at(jat - 1, iat - 1, jadr - 1, iadr - 1, 1) = p[4];
    d.at(jat - 1, iat - 1, jadr - 1, iadr - 1, 2) = p[3];
  }
  const int alk[6] = {3, 11, 19, 37, 55, 87};
  for (int ia = 0; ia < 6; ++ia) {
    const int i = alk[ia] - 1, g = alk[ia] - 2;
    for (int j = 0; j < 94; ++j) {
      const int mj = d.maxci[j];
      for (int ii = 0; ii < d.maxci[i]; ++ii) {
        for (int b = 0; b < mj; ++b) d.at(i, j, ii, b, 0) = d.at(g, j, 0, b, 0);
        for (int b = 0; b < mj; ++b) d.at(j, i, b, ii, 0) = d.at(j, g, b, 0, 0);
      }
      for (int ii = 0; ii < d.maxci[i + 1]; ++ii) {
        for (int b = 0; b < mj; ++b) d.at(i + 1, j, ii, b, 0) = d.at(g, j, 0, b, 0);
        for (int b = 0; b < mj; ++b) d.at(j, i + 1, b, ii, 0) = d.at(j, g, b, 0, 0);
      }
    }
  }
}

inline void ncoord_qmdff(int n, const double* rcov, const int* iz, const double* xyz, double cn_thr,
                         double* cn) {
  const double k1 = 16.0;
  for (int i = 0; i < n; ++i) {
    double xn = 0.0;
    for (int iat = 0; iat < n; ++iat) {
      if (iat == i) continue;
      const double dx = xyz[3 * iat] - xyz[3 * i], dy = xyz[3 * iat + 1] - xyz[3 * i + 1],
                   dz = xyz[3 * iat + 2] - xyz[3 * i + 2];
      const double r2 = dx * dx + dy * dy + dz * dz;
      if (r2 > cn_thr) continue;
      const double r = std::sqrt(r2);
      const double rco = rcov[iz[i] - 1] + rcov[iz[iat] - 1];
      const double rr = rco / r;
      const double damp = 1.0 / (1.0 + std::exp(-k1 * (rr - 1.0)));
      xn = xn + damp;
    }
    cn[i] = xn;
  }
}

inline double getc6(D3Ref& d, int iat, int jat, double nci, double ncj) {
  const double k3 = -4.0;
  double c6mem = -1.0e99, rsum = 0.0, csum = 0.0, r_save = 10000.0;
  for (int i = 0; i < d.maxci[iat - 1]; ++i)
    for (int j = 0; j < d.maxci[jat - 1]; ++j) {
      const double c6 = d.at(iat - 1, jat - 1, i, j, 0);
      if (c6 > 0) {
        const double cn1 = d.at(iat - 1, jat - 1, i, j, 1), cn2 = d.at(iat - 1, jat - 1, i, j, 2);
        const double r = (cn1 - nci) * (cn1 - nci) + (cn2 - ncj) * (cn2 - ncj);  // ** 2 of a real
        if (r < r_save) {
          r_save = r;
          c6mem = c6;
        }
        const double tmp1 = std::exp(k3 * r);
        rsum = rsum + tmp1;
        csum = csum + tmp1 * c6;
      }
    }
  return rsum > 1.0e-99 ? csum / rsum : c6mem;
}

// prepare's pair C6 c6xy (n x n, row-major [i1][i2]) of geometry xyz (bohr)
inline void pair_c6(D3Ref& d, int n, const int* at, const double* xyz, const double* rcov, double* c6xy,
                    double* cn_out) {
  std::vector<double> cn((size_t)n);
  ncoord_qmdff(n, rcov, at, xyz, 5000.0, cn.data());
  for (int i1 = 0; i1 < n; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2) {
      const double c6 = getc6(d, at[i1], at[i2], cn[(size_t)i1], cn[(size_t)i2]);
      c6xy[(size_t)i2 * n + i1] = c6;
      c6xy[(size_t)i1 * n + i2] = c6;
    }
  if (cn_out)
    for (int i = 0; i < n; ++i) cn_out[i] = cn[(size_t)i];
}

}  // namespace orc
