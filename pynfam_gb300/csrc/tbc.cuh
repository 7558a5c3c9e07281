// Finite-range two-body-current (2BC) field: the contraction of the Yukawa part of
// the axial two-body current with the ground-state density matrices,
//
//   Gamma_ac = sum_{db} sum_g  Jz_g(z_a z_b z_c z_d) Jr_g(a b c d) (spin-isospin) rho_db,
//
// the set-up step the reference runs once per operator on the CPU
// (effective_2bc_extfield, pnfam_extfield_2bc.f90:128-465, about 2 h per K component
// at N_sh = 16 with OpenMP) and caches in the .tbc file.
//
// The Gaussian expansion of the Yukawa function (six Gaussians g) separates every
// two-body element into a z part and an (r, phi) part.  The GPU form:
//
//  * host: the 1D Gaussian elements of both directions (the hypergeometric form of
//    HFBTHO's axial element), their derivative variants, the z parts Jz of the
//    current for every (z_a z_b z_c z_d), the polar->Cartesian coefficients, the
//    radial (d, b) terms t = (Omega_b, l_b, l_d, r_b, r_d) with their (z_b, z_d, rho)
//    pairs, and the output elements grouped by their radial quantum numbers
//    (r_a, l_a, r_c, l_c);
//  * k_tbc_z (stage 1): Z[z_a z_c][t][dn, dp, en, ep][14][g] = sum over the pairs of t of
//    Jz * rho (direct and exchange, neutron and proton densities);
//  * k_tbc_field (stage 2): one CTA per radial group.  Its threads compute the (r, phi)
//    current vectors Jr of a chunk of terms once (each a quadruple sum over the
//    Cartesian decompositions of the four polar states, all six Gaussians at once) and
//    then contract them with the Z rows of every element of the group: all z_a, z_c
//    and spins that share the radial quantum numbers reuse one Jr, which the
//    reference recomputes per element.
//
// The per-item arithmetic is in __host__ __device__ functions (TBC_HD) so that it is
// the same code on both sides of any check; the kernels are compiled only by nvcc.
//
// Element order, the pieces (c3d, c3e, c4d, c4e, cpd, cpe with the LECs stripped:
// c3 = 1, c4 + 1/4 = 1) and the spin-sorted layout follow the .tbc file
// (pnfam_storage.f90:488-560, pnfam_extfield_2bc.f90:901-913).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#ifdef __CUDACC__
#define TBC_HD __host__ __device__
#else
#define TBC_HD
#endif

namespace tbc {

constexpr int NG = 6;     // Gaussians of the Yukawa fit
constexpr int NC = 14;    // spatial pieces of the current
constexpr int NCG = NC * NG;
constexpr int NQ = 4;     // Z products: direct n, direct p, exchange n, exchange p
enum { RKP, RKZ, RKM, RPZ, RPM, RZM, R0P, R0Z, R0M, RP0, RZ0, RM0, RPZ2, RZM2 };

// physical constants (pnfam_constants.f90:36-67)
constexpr double PI = 3.141592653589793238462643;
constexpr double HBARC = 197.3269718;
constexpr double MN = 939.0;
constexpr double FPI = 92.4;
constexpr double MPI = 138.04;

// exp(-x)/x = sum_g b_g exp(-a_g x^2) (pnfam_spatial_mtxels.f90:52-55)
static const double Y0_A[NG] = {34.0, 6.60, 1.44, 0.38, 0.15, 0.13};
static const double Y0_B[NG] = {6.79, 2.41, 0.786, 0.241, -0.062, 0.078};

// r-direction tables by (derivatives on the Gaussian, 2i p of particle 1/2)
enum { X00, X10, X20, X11, X12, X01, X02, NXTAB };

// ---------------------------------------------------------------------------------
// device-side view of the prepared tables
// ---------------------------------------------------------------------------------
struct View {
  int K, use_p, bminus;
  int nzx;                    // z of the basis: 0..nzx
  int nrl;                    // r tables: indices 0..nrl (= max 2 n_r + l)
  const double* jz;           // [(nzx+1)^4][NC][NG]
  const double* xr;           // [NXTAB][(nrl+1)^4][NG]
  const double* cp;           // Cp2c [nr <= nrl/2][l + nrl][ny <= nrl]
  int nt;                     // radial (d, b) terms
  const int* tq;              // [nt][5]: Omega_b - 1/2, nl_b, nl_d, r_b, r_d
  const int* poff;            // [nt+1] pairs of term t
  const int* pz;              // [npairs][2] z_b, z_d
  const double* prho;         // [npairs][2] rho_n, rho_p (half of rk)
  int ngroups;
  const int* gq;              // [ngroups][4] r_a, l_a, r_c, l_c
  const int* goff;            // [ngroups+1] elements of each group
  const int* el;              // [nelem][4] z_a, z_c, s_a, s_c
  double* zbuf;               // [(nzx+1)^2][nt][NQ][NC][NG]
  double* acc;                // [nelem][6]
};

TBC_HD inline size_t idx4(int n1, int a, int b, int c, int d) {
  return (((size_t)a * n1 + b) * n1 + c) * n1 + d;
}

TBC_HD inline double cp2c_at(const View& v, int n, int l, int ny) {
  const int L = v.nrl, NY = v.nrl + 1;
  return v.cp[((size_t)n * (2 * L + 1) + (l + L)) * NY + ny];
}

// (r, phi) element with x derivatives only (MatrixElement_radx): the quadruple sum
// over the Cartesian decompositions n = nx + ny of the four polar states; terms of
// odd total ny vanish.  out[g] += scale * value.
TBC_HD inline void radx6(const View& v, int tab, int ni, int li, int nj, int lj, int nk, int lk, int nl, int ll,
                         double scale, double* out) {
  const int n1 = v.nrl + 1;
  const double* X = v.xr + (size_t)tab * n1 * n1 * n1 * n1 * NG;
  const double* Y = v.xr + (size_t)X00 * n1 * n1 * n1 * n1 * NG;
  const int Ai = 2 * ni + (li < 0 ? -li : li), Aj = 2 * nj + (lj < 0 ? -lj : lj);
  const int Ak = 2 * nk + (lk < 0 ? -lk : lk), Al = 2 * nl + (ll < 0 ? -ll : ll);
  double s[NG] = {0, 0, 0, 0, 0, 0};
  for (int yi = 0; yi <= Ai; ++yi) {
    const double ci = cp2c_at(v, ni, li, yi);
    for (int yj = 0; yj <= Aj; ++yj) {
      const double cij = ci * cp2c_at(v, nj, lj, yj);
      for (int yk = 0; yk <= Ak; ++yk) {
        const double cijk = cij * cp2c_at(v, nk, lk, yk);
        for (int yl = (yi + yj + yk) & 1; yl <= Al; yl += 2) {
          const int sgn = (yi + yj + ((yi + yj + yk + yl) >> 1)) & 1;
          const double w = (sgn ? -cijk : cijk) * cp2c_at(v, nl, ll, yl);
          const double* x = X + idx4(n1, Ai - yi, Aj - yj, Ak - yk, Al - yl) * NG;
          const double* y = Y + idx4(n1, yi, yj, yk, yl) * NG;
#pragma unroll
          for (int g = 0; g < NG; ++g) s[g] += w * x[g] * y[g];
        }
      }
    }
  }
#pragma unroll
  for (int g = 0; g < NG; ++g) out[g] += scale * s[g];
}

// imaginary part of the complex (r, phi) element with a y derivative (the
// momentum-dependent pion-pole pieces, MatrixElement_rad_cmplx with dx = 1, py = dip)
TBC_HD inline void radc6_imag(const View& v, int dip, int ni, int li, int nj, int lj, int nk, int lk, int nl, int ll,
                              double* out) {
  const int n1 = v.nrl + 1;
  const double* X = v.xr + (size_t)X10 * n1 * n1 * n1 * n1 * NG;
  const double* Y = v.xr + (size_t)(dip == 1 ? X01 : X02) * n1 * n1 * n1 * n1 * NG;
  const int Ai = 2 * ni + (li < 0 ? -li : li), Aj = 2 * nj + (lj < 0 ? -lj : lj);
  const int Ak = 2 * nk + (lk < 0 ? -lk : lk), Al = 2 * nl + (ll < 0 ? -ll : ll);
  for (int yi = 0; yi <= Ai; ++yi)
    for (int yj = 0; yj <= Aj; ++yj)
      for (int yk = 0; yk <= Ak; ++yk)
        for (int yl = 0; yl <= Al; ++yl) {
          const int e = ((yi + yj - yk - yl) % 4 + 4) % 4;     // i^e
          if (!(e & 1)) continue;
          const double w = (e == 1 ? 1.0 : -1.0) * cp2c_at(v, ni, li, yi) * cp2c_at(v, nj, lj, yj) *
                           cp2c_at(v, nk, lk, yk) * cp2c_at(v, nl, ll, yl);
          const double* x = X + idx4(n1, Ai - yi, Aj - yj, Ak - yk, Al - yl) * NG;
          const double* y = Y + idx4(n1, yi, yj, yk, yl) * NG;
          for (int g = 0; g < NG; ++g) out[g] += w * x[g] * y[g];
        }
}

// (r, phi) part of d_i d_j G, d_i -> 2i P_dip when dip > 0 (MatrixElement_ddGr);
// out[g] = value.  Returns false where the selection rule makes it vanish.
TBC_HD inline bool ddgr6(const View& v, int ni, int li, int nj, int lj, int nk, int lk, int nl, int ll, int di, int dj,
                         int dip, double* out) {
  for (int g = 0; g < NG; ++g) out[g] = 0.0;
  if (-li - lj + lk + ll + di + dj != 0) return false;
  const double r2 = 1.4142135623730951;
  const int p = dip ? 1 : 0;
  const int s = di + dj;
  // table of d derivatives on the Gaussian with the momentum of particle dip
  auto tab = [&](int d, int pp) {
    if (pp == 0) return d == 0 ? (int)X00 : d == 1 ? (int)X10 : (int)X20;
    if (d == 1) return pp == 1 ? (int)X11 : (int)X12;
    return pp == 1 ? (int)X01 : (int)X02;
  };
  if (di == 0 && dj == 0) {
    radx6(v, X00, ni, li, nj, lj, nk, lk, nl, ll, 1.0, out);
  } else if (s == 2 || s == -2) {
    radx6(v, tab(2 - p, dip), ni, li, nj, lj, nk, lk, nl, ll, 2.0, out);
  } else if (s == 1 || s == -1) {
    if (dj == 0) radx6(v, tab(1 - p, dip), ni, li, nj, lj, nk, lk, nl, ll, -s * r2, out);
    else radx6(v, X10, ni, li, nj, lj, nk, lk, nl, ll, -s * r2, out);
  } else {
    radx6(v, tab(2 - p, dip), ni, li, nj, lj, nk, lk, nl, ll, -1.0, out);
    if (dip) radc6_imag(v, dip, ni, li, nj, lj, nk, lk, nl, ll, out);
  }
  return true;
}

// (r, phi) part of the current's 14 pieces for one K (calc_Jr_opt):
// J[c * NG + g].  a, b, c, d = (n, l) of the four states.
TBC_HD inline void jr_vec(const View& v, int na, int la, int nb, int lb, int nc, int lc, int nd, int ld, double* J) {
  for (int i = 0; i < NCG; ++i) J[i] = 0.0;
  const int K = v.K;
  double* o;
#define TBC_R(piece, di, dj, dip) \
  o = J + (piece) * NG;           \
  ddgr6(v, na, la, nb, lb, nc, lc, nd, ld, di, dj, dip, o)
  if (v.use_p) {
    TBC_R(R0P, K, -1, 1); TBC_R(R0Z, K, 0, 1); TBC_R(R0M, K, +1, 1);
    TBC_R(RP0, K, -1, 2); TBC_R(RZ0, K, 0, 2); TBC_R(RM0, K, +1, 2);
  }
  if (K == 1) {
    TBC_R(RKP, +1, -1, 0); TBC_R(RKZ, +1, 0, 0); TBC_R(RKM, +1, +1, 0);
    TBC_R(RPZ, 0, 0, 0);
    for (int g = 0; g < NG; ++g) {
      J[RPM * NG + g] = J[RKZ * NG + g];
      J[RZM * NG + g] = J[RKM * NG + g];
      J[RPZ2 * NG + g] = J[RKP * NG + g];
    }
  } else if (K == 0) {
    TBC_R(RKP, 0, -1, 0); TBC_R(RKZ, 0, 0, 0); TBC_R(RKM, +1, 0, 0);
    TBC_R(RPM, +1, -1, 0);
    for (int g = 0; g < NG; ++g) {
      J[RPZ * NG + g] = J[RKP * NG + g];
      J[RZM * NG + g] = J[RKM * NG + g];
    }
  } else {
    TBC_R(RKP, -1, -1, 0); TBC_R(RKZ, 0, -1, 0); TBC_R(RKM, +1, -1, 0);
    TBC_R(RZM, 0, 0, 0);
    for (int g = 0; g < NG; ++g) {
      J[RPZ * NG + g] = J[RKP * NG + g];
      J[RPM * NG + g] = J[RKZ * NG + g];
      J[RZM2 * NG + g] = J[RKM * NG + g];
    }
  }
#undef TBC_R
}

// ---------------------------------------------------------------------------------
// spin-isospin contraction of one term: the six pieces from the four products
// P[q][c] (q = dn, dp, en, ep; the second d_i d_j Y0 pieces already folded into rpz
// and rzm) for the spins (s_a, s_c) of the element and (s_d, s_b) of the term
// (calc_gam_sep with the gam_Jrs* functions, pnfam_type_extfield_2bc.f90:750-825,
// 869-1463).  sd, sb: -1 or +1; "du" = (s_d, s_b) = (-, +), "ud" = (+, -).
// ---------------------------------------------------------------------------------
TBC_HD inline double jrsa_dir(const double* P, int sa, int sc, int sd, int sb) {
  if (sd + sb == 0) return 0.0;
  if (sa == sc) return 0.5 * sa * P[RKZ];
  return sa > 0 ? P[RKP] : P[RKM];
}
TBC_HD inline double jrsx_dir(const double* P, int sa, int sc, int sd, int sb) {
  const bool du = sd < 0 && sb > 0, ud = sd > 0 && sb < 0, uu = sd + sb > 0;
  if (sa == sc) return du ? -0.5 * sa * P[RPZ] : ud ? 0.5 * sa * P[RZM] : 0.0;
  if (sa > 0) return du ? 0.0 : ud ? P[RPM] : (uu ? 0.5 : -0.5) * P[RPZ];
  return du ? -P[RPM] : ud ? 0.0 : (uu ? -0.5 : 0.5) * P[RZM];
}
TBC_HD inline double jrsxp_dir(const double* P, int sa, int sc, int sd, int sb) {
  const bool du = sd < 0 && sb > 0, ud = sd > 0 && sb < 0, uu = sd + sb > 0;
  if (sa == sc) return du ? P[R0P] : ud ? P[R0M] : 0.5 * sa * P[RZ0] + (uu ? 0.5 : -0.5) * P[R0Z];
  if (du || ud) return 0.0;
  return sa > 0 ? P[RP0] : P[RM0];
}
TBC_HD inline double jrsa_exc(const double* P, int sa, int sc, int sd, int sb) {
  const bool du = sd < 0 && sb > 0, ud = sd > 0 && sb < 0, uu = sd + sb > 0;
  if (sa > 0 && sc > 0) return du ? P[RKP] : ud ? 0.0 : uu ? 0.5 * P[RKZ] : 0.0;
  if (sa < 0 && sc < 0) return du ? 0.0 : ud ? P[RKM] : uu ? 0.0 : -0.5 * P[RKZ];
  if (sa > 0) return du ? 0.0 : ud ? 0.5 * P[RKZ] : uu ? 0.0 : P[RKP];
  return du ? -0.5 * P[RKZ] : ud ? 0.0 : uu ? P[RKM] : 0.0;
}
TBC_HD inline double jrsb_exc(const double* P, int sa, int sc, int sd, int sb) {
  const bool du = sd < 0 && sb > 0, ud = sd > 0 && sb < 0, uu = sd + sb > 0;
  if (sa > 0 && sc > 0) return du ? 0.0 : ud ? P[RKM] : uu ? 0.5 * P[RKZ] : 0.0;
  if (sa < 0 && sc < 0) return du ? P[RKP] : ud ? 0.0 : uu ? 0.0 : -0.5 * P[RKZ];
  if (sa > 0) return du ? 0.0 : ud ? -0.5 * P[RKZ] : uu ? P[RKP] : 0.0;
  return du ? 0.5 * P[RKZ] : ud ? 0.0 : uu ? 0.0 : P[RKM];
}
TBC_HD inline double jrsx_exc(const double* P, int sa, int sc, int sd, int sb) {
  const bool du = sd < 0 && sb > 0, ud = sd > 0 && sb < 0, uu = sd + sb > 0;
  if (sa == sc) {
    if (du) return 0.5 * P[RPZ];
    if (ud) return 0.5 * P[RZM];
    if (sa > 0) return uu ? 0.0 : P[RPM];
    return uu ? -P[RPM] : 0.0;
  }
  if (du || ud) return 0.0;
  return sa > 0 ? -0.5 * P[RPZ] : -0.5 * P[RZM];
}
TBC_HD inline double jrsxp_exc(const double* P, int sa, int sc, int sd, int sb) {
  const bool du = sd < 0 && sb > 0, ud = sd > 0 && sb < 0, uu = sd + sb > 0;
  if (sa > 0 && sc > 0) return du ? P[RP0] : ud ? P[R0M] : uu ? 0.5 * (P[RZ0] + P[R0Z]) : 0.0;
  if (sa < 0 && sc < 0) return du ? P[R0P] : ud ? P[RM0] : uu ? 0.0 : -0.5 * (P[RZ0] + P[R0Z]);
  if (sa > 0) return du ? 0.0 : ud ? 0.5 * (P[RZ0] - P[R0Z]) : uu ? P[R0P] : P[RP0];
  return du ? 0.5 * (P[R0Z] - P[RZ0]) : ud ? 0.0 : uu ? P[RM0] : P[R0M];
}

// gam[0..5] += sign * pieces of one term.  zrow: [NQ][NC][NG] of the element's
// (z_a, z_c) and the term; jd, je: direct and exchange (r, phi) currents [NC][NG].
TBC_HD inline void contract_term(const double* zrow, const double* jd, const double* je, int sa, int sc, int sd,
                                 int sb, int bminus, double sign, double* gam) {
  double P[NQ][NC];
  for (int q = 0; q < NQ; ++q) {
    const double* z = zrow + q * NCG;
    const double* j = q < 2 ? jd : je;
    for (int c = 0; c < NC; ++c) {
      double s = 0.0;
#pragma unroll
      for (int g = 0; g < NG; ++g) s += z[c * NG + g] * j[c * NG + g];
      P[q][c] = s;
    }
    P[q][RPZ] += P[q][RPZ2];
    P[q][RZM] += P[q][RZM2];
  }
  const double a_dn = jrsa_dir(P[0], sa, sc, sd, sb), a_dp = jrsa_dir(P[1], sa, sc, sd, sb);
  const double x_dn = jrsx_dir(P[0], sa, sc, sd, sb), x_dp = jrsx_dir(P[1], sa, sc, sd, sb);
  const double xp_dn = jrsxp_dir(P[0], sa, sc, sd, sb), xp_dp = jrsxp_dir(P[1], sa, sc, sd, sb);
  const double a_en = jrsa_exc(P[2], sa, sc, sd, sb), b_en = jrsb_exc(P[2], sa, sc, sd, sb);
  const double a_ep = jrsa_exc(P[3], sa, sc, sd, sb), b_ep = jrsb_exc(P[3], sa, sc, sd, sb);
  const double x_e = jrsx_exc(P[2], sa, sc, sd, sb) + jrsx_exc(P[3], sa, sc, sd, sb);
  const double xp_e = jrsxp_exc(P[2], sa, sc, sd, sb) + jrsxp_exc(P[3], sa, sc, sd, sb);
  const double h = bminus ? 0.5 : -0.5;
  gam[0] += sign * (a_dn + a_dp);
  gam[1] += sign * (bminus ? -a_en - b_ep : -b_en - a_ep);
  gam[2] += sign * (h * (x_dn - x_dp));
  gam[3] += sign * (-0.5 * x_e);
  gam[4] += sign * (h * (xp_dn - xp_dp));
  gam[5] += sign * (-0.5 * xp_e);
}

// the two (r, phi) branches of term t for an element of radial quantum numbers
// (ra, la, rc, lc): branch 0 with (l_b, l_d), branch 1 with the time-reversed
// (-l_b, -l_d) (pnfam_extfield_2bc.f90:349-418).  Returns false where the branch
// does not contribute; otherwise the spins (s_d, s_b) and the sign of the term.
TBC_HD inline bool term_branch(const View& v, int t, int br, int la, int lc, int* lb, int* ld, int* sd, int* sb,
                               double* sign) {
  const int* q = v.tq + 5 * t;
  const int ob = q[0], nlb = q[1], nld = q[2];
  const int l_b = ob + nlb, l_d = ob + nld;
  const int s_b = 1 - 2 * nlb, s_d = 1 - 2 * nld;
  const int K = v.K;
  if (br == 0) {
    const int x = la + l_b - lc - l_d;
    if (x != K + 1 && x != K && x != K - 1) return false;
    *lb = l_b; *ld = l_d; *sd = s_d; *sb = s_b; *sign = 1.0;
  } else {
    const int x = la - l_b - lc + l_d;
    if (x != K + 1 && x != K && x != K - 1) return false;
    *lb = -l_b; *ld = -l_d; *sd = -s_d; *sb = -s_b; *sign = (s_d + s_b == 0) ? -1.0 : 1.0;
  }
  return true;
}

// ---------------------------------------------------------------------------------
// host-side preparation
// ---------------------------------------------------------------------------------
struct Input {
  int ntx, nbx;
  const int* block_size;             // [nbx]
  const int *nz, *nr, *nl, *ns;      // [ntx] HFBTHO order
  double bz, bp;
  const double* rk_n;                // per block [d*d] column-major, concatenated
  const double* rk_p;
  int K, beta_minus, use_p;
  const int* op_cols;                // [2 nbx] 0-based column block, -1 empty
  const long long* op_offsets;       // [2 nbx]
  long long nxy;
};

struct Prepared {
  int nzx = 0, nrx = 0, nrl = 0, nox = 0;
  std::vector<double> jz, xr, cp;
  std::vector<int> tq, poff, pz;
  std::vector<double> prho;
  std::vector<int> gq, goff, el;
  std::vector<long long> out_index;  // [nelem] flat index of the element (spin-sorted)
  std::vector<double> out_sign;      // [nelem] sign_a * sign_c
  int max_group = 0;
};

struct Math1D {
  static constexpr int GMAX = 200;     // Gamma(m / 2) for |m| <= GMAX, m odd
  std::vector<double> fact, ghalf;
  Math1D() {
    fact.resize(171);
    fact[0] = 1.0;
    for (int i = 1; i <= 170; ++i) fact[i] = i * fact[i - 1];
    ghalf.assign(2 * GMAX + 1, 0.0);
    for (int m = -GMAX; m <= GMAX; ++m)
      if (m & 1) ghalf[m + GMAX] = std::tgamma(0.5 * m);
  }
  // Gamma(x) of a half-integer x (the arguments of the axial element)
  double gamma_half(double x) const {
    const int m = (int)std::lround(2.0 * x);
    return (m & 1) && m >= -GMAX && m <= GMAX ? ghalf[m + GMAX] : std::tgamma(x);
  }
  double binom(int m, int n) const {
    if (n < 0 || n > m) return 0.0;
    if (n == 0 || n == m) return 1.0;
    if (n == 1 || n == m - 1) return (double)m;
    return n <= m / 2 ? (fact[m] / fact[m - n]) / fact[n] : (fact[m] / fact[n]) / fact[m - n];
  }
  // 2F1(a, b; c; x) for non-positive integers a, b: a terminating series
  double hyp2f1(int a, int b, double c, double x) const {
    const int d = std::abs(std::max(a, b)), e = std::abs(std::min(a, b));
    double s = 0.0, xi = 1.0, up = 1.0;         // x^i and the rising factorial (c)_i
    for (int i = 0; i <= d; ++i) {
      s += binom(d, i) * binom(e, i) * xi * fact[i] / up;
      xi *= x;
      up *= c + i;
    }
    return s;
  }
  double tz(int n1, int n2, int n) const {
    if (n1 > n2) std::swap(n1, n2);
    if (n < n2 - n1 || n > n1 + n2 || ((n - n1 - n2) & 1)) return 0.0;
    const int m1 = (-n1 + n2 + n) / 2, m2 = (n1 - n2 + n) / 2, m3 = (n1 + n2 - n) / 2;
    return (std::sqrt(fact[n2]) / fact[m1]) * (std::sqrt(fact[n]) / fact[m2]) * (std::sqrt(fact[n1]) / fact[m3]);
  }
  // <ni nj| exp(-(x1 - x2)^2 / mu^2) |nk nl> of 1D oscillator functions of length b:
  // the hypergeometric form (Younes 2009, Eq. D.12), summed over the shorter of the
  // two Talmi-like expansions
  double me(int ni, int nj, int nk, int nl, double mu, double b) const {
    int s1 = (nj + nl - std::abs(nj - nl)) / 2 + 1, s2 = (ni + nk - std::abs(ni - nk)) / 2 + 1;
    if (s1 == s2) { s1 = std::min(ni, nk); s2 = std::min(nj, nl); }
    int i = ni, j = nj, k = nk, l = nl;
    if (s1 > s2) { i = nj; j = ni; k = nl; l = nk; }
    const double z = 1.0 + mu * mu / (2.0 * b * b);
    double v = 0.0;
    for (int n = std::abs(j - l); n <= j + l; n += 2) {
      if ((i + k + n) & 1) break;
      const double xi = (i + k + n + 1) * 0.5;
      const double fbar = gamma_half(xi - i) * gamma_half(xi - k) * gamma_half(xi - n) /
                          (std::pow(z, xi) * std::sqrt(fact[i] * fact[k] * fact[n])) *
                          hyp2f1(-i, -k, n + 1 - xi, 1 - z);
      v += tz(j, l, n) * fbar;
    }
    return mu / (std::sqrt(2.0 * PI * PI * PI) * b) * v;
  }
  // polar (n, k) -> Cartesian (nx, ny) coefficient of 2D oscillator functions
  double cp2c(int n, int k, int ny) const {
    const int ak = std::abs(k);
    if (ny < 0 || ny > 2 * n + ak) return 0.0;
    const int nx = 2 * n + ak - ny;
    const double a = ((n & 1) ? -1.0 : 1.0) * std::pow(2.0, -n - ak * 0.5) * std::sqrt(fact[n + ak]) *
                     (std::sqrt(fact[n]) / (std::sqrt(fact[nx]) * std::sqrt(fact[ny])));
    const int h = (ak - k) / 2;
    double s = 0.0;
    for (int q = 0; q <= std::min(ny, n + h); ++q) s += binom(nx, n - q + h) * binom(ny, q) * (((ny - q) & 1) ? -1.0 : 1.0);
    return a * s;
  }
};

// dense 1D tables of one direction: [NG][n1^4] of the bare Gaussian element
// (times the Gaussian's prefactor for z), for indices 0..nmax
struct Dir1D {
  int n1;
  double pd1, pd2;                    // derivative prefactors 1/(b sqrt 2), 1/(2 b^2)
  std::vector<double> t;              // [n1^4][NG]
  double at(int a, int b, int c, int d, int g) const {
    if (a < 0 || b < 0 || c < 0 || d < 0 || a >= n1 || b >= n1 || c >= n1 || d >= n1) return 0.0;
    return t[idx4(n1, a, b, c, d) * NG + g];
  }
  // d-th derivative of a 1D oscillator function: up to three (n', coefficient)
  int deriv(int n, int d, int* nn, double* cc) const {
    if (d == 0) { nn[0] = n; cc[0] = 1.0; return 1; }
    if (d == 1) {
      nn[0] = n + 1; cc[0] = -std::sqrt((double)(n + 1)) * pd1;
      if (n >= 1) { nn[1] = n - 1; cc[1] = std::sqrt((double)n) * pd1; return 2; }
      return 1;
    }
    nn[0] = n + 2; cc[0] = std::sqrt((double)((n + 1) * (n + 2))) * pd2;
    nn[1] = n; cc[1] = -(2.0 * n + 1.0) * pd2;
    if (n >= 2) { nn[2] = n - 2; cc[2] = std::sqrt((double)(n * (n - 1))) * pd2; return 3; }
    return 2;
  }
  void dho(int ni, int nj, int nk, int nl, int di, int dj, int dk, int dl, double* out) const {
    int a[3], b[3], c[3], d[3];
    double ca[3], cb[3], cc[3], cd[3];
    const int na = deriv(ni, di, a, ca), nb = deriv(nj, dj, b, cb), nc = deriv(nk, dk, c, cc), nd = deriv(nl, dl, d, cd);
    for (int g = 0; g < NG; ++g) out[g] = 0.0;
    for (int l = 0; l < nd; ++l)
      for (int k = 0; k < nc; ++k)
        for (int j = 0; j < nb; ++j)
          for (int i = 0; i < na; ++i) {
            if ((a[i] + b[j] + c[k] + d[l]) & 1) continue;
            const double w = ca[i] * cb[j] * cc[k] * cd[l];
            for (int g = 0; g < NG; ++g) out[g] += at(a[i], b[j], c[k], d[l], g) * w;
          }
  }
  // d derivatives on the Gaussian, or 2i p of particle p (1 or 2): by parts onto the
  // oscillator functions
  void me_dp(int ni, int nj, int nk, int nl, int d, int p, double* out) const {
    for (int g = 0; g < NG; ++g) out[g] = 0.0;
    const int par = ni + nj + nk + nl + d;
    if (p == 0) {
      if (par & 1) return;
    } else {
      if (!(par & 1)) return;
      if (p == 1 && ni == nk) return;
      if (p == 2 && nj == nl) return;
    }
    double u[NG], w[NG];
    auto acc = [&](const double* x, double s) { for (int g = 0; g < NG; ++g) out[g] += s * x[g]; };
    if (d == 0 && p == 0) { for (int g = 0; g < NG; ++g) out[g] = at(ni, nj, nk, nl, g); return; }
    if (d == 1 && p == 0) { dho(ni, nj, nk, nl, 1, 0, 0, 0, u); dho(ni, nj, nk, nl, 0, 0, 1, 0, w); acc(u, -1); acc(w, -1); return; }
    if (d == 2 && p == 0) {
      dho(ni, nj, nk, nl, 2, 0, 0, 0, u); acc(u, 1); dho(ni, nj, nk, nl, 0, 0, 2, 0, u); acc(u, 1);
      dho(ni, nj, nk, nl, 1, 0, 1, 0, w); acc(w, 2); return;
    }
    if (d == 1 && p == 1) { dho(ni, nj, nk, nl, 0, 0, 2, 0, u); dho(ni, nj, nk, nl, 2, 0, 0, 0, w); acc(u, -1); acc(w, 1); return; }
    if (d == 1 && p == 2) { dho(ni, nj, nk, nl, 0, 0, 0, 2, u); dho(ni, nj, nk, nl, 0, 2, 0, 0, w); acc(u, 1); acc(w, -1); return; }
    if (d == 0 && p == 1) { dho(ni, nj, nk, nl, 0, 0, 1, 0, u); dho(ni, nj, nk, nl, 1, 0, 0, 0, w); acc(u, 1); acc(w, -1); return; }
    if (d == 0 && p == 2) { dho(ni, nj, nk, nl, 0, 0, 0, 1, u); dho(ni, nj, nk, nl, 0, 1, 0, 0, w); acc(u, 1); acc(w, -1); return; }
  }
};

// run f(i) for i in [0, n) on the host's cores (each i written by one thread)
template <class F>
inline void host_parallel(int n, F f) {
  const int nt = std::max(1, std::min(n, (int)std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (int w = 0; w < nt; ++w)
    th.emplace_back([=]() {
      for (int i = w; i < n; i += nt) f(i);
    });
  for (auto& t : th) t.join();
}

inline Dir1D make_dir(const Math1D& m, int nmax, double b, const double* mu, const double* pf) {
  Dir1D d;
  d.n1 = nmax + 1;
  d.pd1 = 1.0 / (b * 1.4142135623730951);
  d.pd2 = 1.0 / (b * b * 2.0);
  d.t.assign((size_t)d.n1 * d.n1 * d.n1 * d.n1 * NG, 0.0);
  const int n1 = d.n1;
  double* t = d.t.data();
  host_parallel(n1 * n1, [&](int ab) {
    const int a = ab / n1, bb = ab % n1;
    for (int c = 0; c < n1; ++c)
      for (int dd = 0; dd < n1; ++dd) {
        if ((a + bb + c + dd) & 1) continue;
        for (int g = 0; g < NG; ++g) {
          double v = m.me(a, bb, c, dd, mu[g], b);
          if (pf) v *= pf[g];
          t[idx4(n1, a, bb, c, dd) * NG + g] = v;
        }
      }
  });
  return d;
}

// z part of d_i d_j G (MatrixElement_ddGz)
inline void ddgz(const Dir1D& z, int ni, int nj, int nk, int nl, int di, int dj, int dip, double* out) {
  const int p = dip ? 1 : 0, s = di + dj;
  if (di == 0 && dj == 0) z.me_dp(ni, nj, nk, nl, 2 - p, dip, out);
  else if (s == 0 || s == 2 || s == -2) z.me_dp(ni, nj, nk, nl, 0, 0, out);
  else if (di == 0) z.me_dp(ni, nj, nk, nl, 1 - p, dip, out);
  else z.me_dp(ni, nj, nk, nl, 1, 0, out);
}

// z part of the current's 14 pieces for one K with the LEC-stripped prefactors
// (calc_Jz_opt, pnfam_type_extfield_2bc.f90:182-288; c3 = 1, c4 + 1/4 = 1)
inline void jz_vec(const Dir1D& z, int K, int use_p, int ni, int nj, int nk, int nl, double* J) {
  const double r2 = 1.4142135623730951;
  const double caux = HBARC * HBARC * HBARC / (2.0 * MN * FPI * FPI);
  const double c3r = caux * (4.0 * r2), c38 = caux * 8.0;
  const double cy0p = caux * 4.0;
  const double yr = cy0p * (2.0 * r2), y2 = cy0p * 2.0, y4 = cy0p * 4.0;
  for (int i = 0; i < NCG; ++i) J[i] = 0.0;
  double a[NG], b[NG], c[NG];
  auto put = [&](int piece, double s, const double* x) { for (int g = 0; g < NG; ++g) J[piece * NG + g] = s * x[g]; };
  if (use_p) {
    ddgz(z, ni, nj, nk, nl, K, -1, 1, a); put(R0P, caux * r2, a);
    ddgz(z, ni, nj, nk, nl, K, 0, 1, a); put(R0Z, caux * 2.0, a);
    ddgz(z, ni, nj, nk, nl, K, +1, 1, a); put(R0M, -caux * r2, a);
    ddgz(z, ni, nj, nk, nl, K, -1, 2, a); put(RP0, caux * r2, a);
    ddgz(z, ni, nj, nk, nl, K, 0, 2, a); put(RZ0, caux * 2.0, a);
    ddgz(z, ni, nj, nk, nl, K, +1, 2, a); put(RM0, -caux * r2, a);
  }
  ddgz(z, ni, nj, nk, nl, +1, -1, 0, a);   // d+ d-  (= d+ d+ = d- d-)
  ddgz(z, ni, nj, nk, nl, 0, 0, 0, b);     // d0 d0
  ddgz(z, ni, nj, nk, nl, 0, -1, 0, c);    // d0 d-  (= d+ d0)
  if (K == 1) {
    put(RKP, -c3r, a); put(RKZ, -c38, c); put(RKM, c3r, a);
    put(RPZ, yr, b); put(RPM, -y2, c); put(RZM, -yr, a); put(RPZ2, -yr, a);
  } else if (K == 0) {
    put(RKP, -c3r, c); put(RKZ, -c38, b); put(RKM, c3r, c);
    put(RPZ, yr, c); put(RPM, -y4, a); put(RZM, -yr, c);
  } else {
    put(RKP, -c3r, a); put(RKZ, -c38, c); put(RKM, c3r, a);
    put(RPZ, yr, a); put(RPM, -y2, c); put(RZM, -yr, b); put(RZM2, yr, a);
  }
}

inline std::string prepare(const Input& in, Prepared& P) {
  if (in.K < -1 || in.K > 1) return "the two-body current needs K in {-1, 0, 1}";
  const int ntx = in.ntx, nbx = in.nbx;
  if (ntx <= 0 || nbx <= 0) return "empty basis";
  std::vector<int> db(2 * nbx), isstart(2 * nbx), ib_itx(2 * ntx);
  int tot = 0;
  for (int i = 0; i < 2 * nbx; ++i) { db[i] = in.block_size[i % nbx]; isstart[i] = tot; tot += db[i]; }
  if (tot != 2 * ntx) return "block sizes do not add up to the basis";
  for (int i = 0, s = 0; i < 2 * nbx; ++i)
    for (int j = 0; j < db[i]; ++j) ib_itx[s++] = i;
  int nlx = 0;
  for (int t = 0; t < ntx; ++t) {
    if (in.nl[t] < 0 || in.nz[t] < 0 || in.nr[t] < 0 || (in.ns[t] != 1 && in.ns[t] != -1)) return "bad quantum numbers";
    P.nzx = std::max(P.nzx, in.nz[t]); P.nrx = std::max(P.nrx, in.nr[t]); nlx = std::max(nlx, in.nl[t]);
    P.nrl = std::max(P.nrl, 2 * in.nr[t] + in.nl[t]);
    P.nox = std::max(P.nox, in.nl[t] + (in.ns[t] + 1) / 2 - 1);
  }
  // state index of (z, r, l, s)
  const int NZ = P.nzx + 1, NR = P.nrx + 1, NLL = nlx + 2;
  std::vector<int> index((size_t)NZ * NR * NLL * 2, -1);
  auto sidx = [&](int z, int r, int l, int s) -> int {
    if (z < 0 || z >= NZ || r < 0 || r >= NR || l < 0 || l >= NLL) return -1;
    return index[(((size_t)z * NR + r) * NLL + l) * 2 + (s > 0 ? 1 : 0)];
  };
  for (int t = 0; t < ntx; ++t)
    index[(((size_t)in.nz[t] * NR + in.nr[t]) * NLL + in.nl[t]) * 2 + (in.ns[t] > 0 ? 1 : 0)] = t;

  // Gaussian widths and prefactors of Y0(x) = exp(-m_pi x) / (4 pi x)
  double mu[NG], pf[NG];
  const double m = MPI / HBARC;
  for (int g = 0; g < NG; ++g) { mu[g] = (1.0 / std::sqrt(Y0_A[g])) / m; pf[g] = Y0_B[g] * m * 0.25 / PI; }
  Math1D M;
  const Dir1D dz = make_dir(M, P.nzx + 2, in.bz, mu, pf);
  const Dir1D dr = make_dir(M, P.nrl + 2, in.bp, mu, nullptr);

  // z parts of the current for every (z_a, z_b, z_c, z_d)
  P.jz.assign((size_t)NZ * NZ * NZ * NZ * NCG, 0.0);
  double* jzp = P.jz.data();
  host_parallel(NZ * NZ, [&](int ab) {
    const int a = ab / NZ, b = ab % NZ;
    for (int c = 0; c < NZ; ++c)
      for (int d = 0; d < NZ; ++d) jz_vec(dz, in.K, in.use_p, a, b, c, d, jzp + idx4(NZ, a, b, c, d) * NCG);
  });
  // r tables with derivatives, indices 0..nrl
  const int n1 = P.nrl + 1;
  const size_t tsz = (size_t)n1 * n1 * n1 * n1 * NG;
  P.xr.assign(NXTAB * tsz, 0.0);
  const int dtab[NXTAB][2] = {{0, 0}, {1, 0}, {2, 0}, {1, 1}, {1, 2}, {0, 1}, {0, 2}};
  double* xrp = P.xr.data();
  for (int k = 0; k < NXTAB; ++k) {
    if (k >= X11 && !in.use_p) break;
    host_parallel(n1 * n1, [&](int ab) {
      const int a = ab / n1, b = ab % n1;
      for (int c = 0; c < n1; ++c)
        for (int d = 0; d < n1; ++d) dr.me_dp(a, b, c, d, dtab[k][0], dtab[k][1], xrp + k * tsz + idx4(n1, a, b, c, d) * NG);
    });
  }
  // polar -> Cartesian coefficients, n <= nrl/2, |l| <= nrl, ny <= nrl
  const int L = P.nrl;
  P.cp.assign((size_t)(L / 2 + 1) * (2 * L + 1) * (L + 1), 0.0);
  for (int n = 0; n <= L / 2; ++n)
    for (int l = -L; l <= L; ++l)
      for (int ny = 0; ny <= L; ++ny)
        if (2 * n + std::abs(l) <= L) P.cp[((size_t)n * (2 * L + 1) + (l + L)) * (L + 1) + ny] = M.cp2c(n, l, ny);

  // the (k, r, l, s) groups of the basis with their z lists, as HFBTHO's base builds
  // them for finite-range forces: z in even, then odd z + l order
  auto zlist = [&](int r, int l, int s) {
    std::vector<int> zs;
    for (int ip = 0; ip < 2; ++ip)
      for (int z = 0; z < NZ; ++z)
        if (((z + l) & 1) == ip && sidx(z, r, l, s) >= 0) zs.push_back(z);
    return zs;
  };
  // radial (d, b) terms in the reference's loop order and their (z_b, z_d) pairs
  // (the stage-1 loops over groups with k_b = k_d, pnfam_extfield_2bc.f90:188-255)
  std::vector<size_t> boff(nbx);
  for (int i = 0, o = 0; i < nbx; ++i) { boff[i] = o; o += db[i] * db[i]; }
  P.poff.push_back(0);
  for (int ob = 0; ob <= P.nox; ++ob)
    for (int nlb = 0; nlb < 2; ++nlb)
      for (int nld = 0; nld < 2; ++nld) {
        const int lb = ob + nlb, ld = ob + nld, sb = 1 - 2 * nlb, sd = 1 - 2 * nld;
        for (int rb = 0; rb <= P.nrx; ++rb) {
          if (2 * rb + lb > P.nrl) continue;
          for (int rd = 0; rd <= P.nrx; ++rd) {
            if (2 * rd + ld > P.nrl) continue;
            P.tq.insert(P.tq.end(), {ob, nlb, nld, rb, rd});
            for (int zb : zlist(rb, lb, sb)) {
              const int jb = sidx(zb, rb, lb, sb);
              const int ibb = ib_itx[jb], inb = jb - isstart[ibb];
              for (int zd : zlist(rd, ld, sd)) {
                const int jd = sidx(zd, rd, ld, sd);
                if (ib_itx[jd] != ibb) continue;
                const int ind = jd - isstart[ibb];
                const size_t e = boff[ibb] + (size_t)ind + (size_t)inb * db[ibb];
                P.pz.push_back(zb); P.pz.push_back(zd);
                P.prho.push_back(in.rk_n[e] * 0.5); P.prho.push_back(in.rk_p[e] * 0.5);
              }
            }
            P.poff.push_back((int)(P.pz.size() / 2));
          }
        }
      }
  // output elements grouped by (r_a, l_a, r_c, l_c); the flat index is the one after
  // the spin sort of every block (spin-up states first, then spin-down, each in
  // HFBTHO order)
  std::vector<int> spos(2 * ntx);
  for (int ib = 0; ib < 2 * nbx; ++ib) {
    int k = 0;
    for (int pass = 0; pass < 2; ++pass)
      for (int j = 0; j < db[ib]; ++j) {
        const int st = isstart[ib] + j;
        const int s = st < ntx ? in.ns[st] : -in.ns[st - ntx];
        if ((pass == 0) == (s > 0)) spos[st] = k++;
      }
  }
  std::map<std::tuple<int, int, int, int>, std::vector<int>> groups;
  std::vector<int> els;
  std::vector<long long> oidx;
  std::vector<double> osgn;
  for (int a = 0; a < 2 * ntx; ++a) {
    const int ia = a < ntx ? a : a - ntx, atr = a < ntx ? 1 : -1;
    const int iba = ib_itx[a], ibc = in.op_cols[iba];
    if (ibc < 0) continue;
    for (int c = isstart[ibc]; c < isstart[ibc] + db[ibc]; ++c) {
      const int ic = c < ntx ? c : c - ntx, ctr = c < ntx ? 1 : -1;
      const int e = (int)(els.size() / 4);
      els.insert(els.end(), {in.nz[ia], in.nz[ic], in.ns[ia] * atr, in.ns[ic] * ctr});
      oidx.push_back(in.op_offsets[iba] + spos[a] + (long long)spos[c] * db[iba]);
      const double sa = (a >= ntx && in.ns[ia] < 0) ? -1.0 : 1.0, sc = (c >= ntx && in.ns[ic] < 0) ? -1.0 : 1.0;
      osgn.push_back(sa * sc);
      groups[std::make_tuple(in.nr[ia], in.nl[ia] * atr, in.nr[ic], in.nl[ic] * ctr)].push_back(e);
    }
  }
  P.goff.push_back(0);
  for (auto& kv : groups) {
    P.gq.insert(P.gq.end(), {std::get<0>(kv.first), std::get<1>(kv.first), std::get<2>(kv.first), std::get<3>(kv.first)});
    for (int e : kv.second) {
      P.el.insert(P.el.end(), {els[4 * e], els[4 * e + 1], els[4 * e + 2], els[4 * e + 3]});
      P.out_index.push_back(oidx[e]);
      P.out_sign.push_back(osgn[e]);
    }
    P.max_group = std::max(P.max_group, (int)kv.second.size());
    P.goff.push_back((int)P.out_index.size());
  }
  for (long long x : P.out_index)
    if (x < 0 || x >= in.nxy) return "operator block structure does not match the basis";
  return "";
}

inline View view_of(const Input& in, const Prepared& P) {
  View v;
  v.K = in.K; v.use_p = in.use_p; v.bminus = in.beta_minus;
  v.nzx = P.nzx; v.nrl = P.nrl;
  v.jz = P.jz.data(); v.xr = P.xr.data(); v.cp = P.cp.data();
  v.nt = (int)(P.tq.size() / 5); v.tq = P.tq.data(); v.poff = P.poff.data(); v.pz = P.pz.data(); v.prho = P.prho.data();
  v.ngroups = (int)(P.gq.size() / 4); v.gq = P.gq.data(); v.goff = P.goff.data(); v.el = P.el.data();
  v.zbuf = nullptr; v.acc = nullptr;
  return v;
}

// the six pieces [6][nxy] from the per-element sums acc [nelem][6]
inline void scatter(const Prepared& P, const double* acc, long long nxy, double* pieces) {
  for (size_t i = 0; i < (size_t)6 * nxy; ++i) pieces[i] = 0.0;
  for (size_t e = 0; e < P.out_index.size(); ++e)
    for (int k = 0; k < 6; ++k) pieces[(size_t)k * nxy + P.out_index[e]] = acc[6 * e + k] * P.out_sign[e];
}

// ---------------------------------------------------------------------------------
// the two stages as per-item functions (one item = one thread of the kernels)
// ---------------------------------------------------------------------------------
// Z[zac][t][q][cg] for one (zac, t, cg)
TBC_HD inline void stage1_item(const View& v, int zac, int t, int cg) {
  const int NZ = v.nzx + 1, za = zac / NZ, zc = zac % NZ;
  double dn = 0, dp = 0, en = 0, ep = 0;
  for (int p = v.poff[t]; p < v.poff[t + 1]; ++p) {
    const int zb = v.pz[2 * p], zd = v.pz[2 * p + 1];
    const double rn = v.prho[2 * p], rp = v.prho[2 * p + 1];
    const double jd = v.jz[idx4(NZ, za, zb, zc, zd) * NCG + cg];
    const double je = v.jz[idx4(NZ, za, zb, zd, zc) * NCG + cg];
    dn += jd * rn; dp += jd * rp; en += je * rn; ep += je * rp;
  }
  double* z = v.zbuf + ((size_t)zac * v.nt + t) * NQ * NCG + cg;
  z[0] = dn; z[NCG] = dp; z[2 * NCG] = en; z[3 * NCG] = ep;
}

// (r, phi) current of one (group, term, branch): the direct (de = 0) or exchange
// (de = 1) one, J [NCG]; false if the branch does not contribute
TBC_HD inline bool stage2_jr(const View& v, int grp, int t, int br, int de, double* J) {
  const int* q = v.gq + 4 * grp;
  const int ra = q[0], la = q[1], rc = q[2], lc = q[3];
  int lb, ld, sd, sb;
  double sign;
  if (!term_branch(v, t, br, la, lc, &lb, &ld, &sd, &sb, &sign)) return false;
  const int rb = v.tq[5 * t + 3], rd = v.tq[5 * t + 4];
  if (de == 0) jr_vec(v, ra, la, rb, lb, rc, lc, rd, ld, J);
  else jr_vec(v, ra, la, rb, lb, rd, ld, rc, lc, J);
  return true;
}

// one element's contribution of (term, branch) with its currents jd, je
TBC_HD inline void stage2_elem(const View& v, int grp, int e, int t, int br, const double* jd, const double* je,
                               double* gam) {
  const int* q = v.gq + 4 * grp;
  int lb, ld, sd, sb;
  double sign;
  term_branch(v, t, br, q[1], q[3], &lb, &ld, &sd, &sb, &sign);
  const int* E = v.el + 4 * e;
  const int zac = E[0] * (v.nzx + 1) + E[1];
  const double* zrow = v.zbuf + ((size_t)zac * v.nt + t) * NQ * NCG;
  contract_term(zrow, jd, je, E[2], E[3], sd, sb, v.bminus, sign, gam);
}

#ifdef __CUDACC__
// stage 1: one thread per (zac, t, cg)
__global__ void k_tbc_z(View v, long long total) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int cg = (int)(i % NCG);
    const long long r = i / NCG;
    stage1_item(v, (int)(r / v.nt), (int)(r % v.nt), cg);
  }
}

constexpr int TBC_TCH = 32;         // terms per chunk
constexpr int TBC_THREADS = 256;    // 8 warps
constexpr size_t TBC_SMEM = sizeof(double) * TBC_TCH * 4 * NCG;

__device__ __forceinline__ void warp_sum6(double* s) {
#pragma unroll
  for (int g = 0; g < NG; ++g)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s[g] += __shfl_xor_sync(0xffffffffu, s[g], o);
}

// radx6 with the 32 lanes of a warp splitting the (ny_i, ny_j, ny_k) combinations;
// every lane returns the full sums.  Called by all lanes with the same arguments.
__device__ void radx6_warp(const View& v, int lane, int tab, int ni, int li, int nj, int lj, int nk, int lk, int nl,
                           int ll, double* s) {
  const int n1 = v.nrl + 1;
  const double* X = v.xr + (size_t)tab * n1 * n1 * n1 * n1 * NG;
  const double* Y = v.xr + (size_t)X00 * n1 * n1 * n1 * n1 * NG;
  const int Ai = 2 * ni + abs(li), Aj = 2 * nj + abs(lj), Ak = 2 * nk + abs(lk), Al = 2 * nl + abs(ll);
  const int n3 = (Ai + 1) * (Aj + 1) * (Ak + 1);
  for (int g = 0; g < NG; ++g) s[g] = 0.0;
  for (int c = lane; c < n3; c += 32) {
    const int yk = c % (Ak + 1), r = c / (Ak + 1), yj = r % (Aj + 1), yi = r / (Aj + 1);
    const double cijk = cp2c_at(v, ni, li, yi) * cp2c_at(v, nj, lj, yj) * cp2c_at(v, nk, lk, yk);
    for (int yl = (yi + yj + yk) & 1; yl <= Al; yl += 2) {
      const int sgn = (yi + yj + ((yi + yj + yk + yl) >> 1)) & 1;
      const double w = (sgn ? -cijk : cijk) * cp2c_at(v, nl, ll, yl);
      const double* x = X + idx4(n1, Ai - yi, Aj - yj, Ak - yk, Al - yl) * NG;
      const double* y = Y + idx4(n1, yi, yj, yk, yl) * NG;
#pragma unroll
      for (int g = 0; g < NG; ++g) s[g] += w * x[g] * y[g];
    }
  }
  warp_sum6(s);
}

// radc6_imag with the lanes of a warp splitting the (ny_i, ny_j, ny_k) combinations
__device__ void radc6_imag_warp(const View& v, int lane, int dip, int ni, int li, int nj, int lj, int nk, int lk,
                                int nl, int ll, double* s) {
  const int n1 = v.nrl + 1;
  const double* X = v.xr + (size_t)X10 * n1 * n1 * n1 * n1 * NG;
  const double* Y = v.xr + (size_t)(dip == 1 ? X01 : X02) * n1 * n1 * n1 * n1 * NG;
  const int Ai = 2 * ni + abs(li), Aj = 2 * nj + abs(lj), Ak = 2 * nk + abs(lk), Al = 2 * nl + abs(ll);
  const int n3 = (Ai + 1) * (Aj + 1) * (Ak + 1);
  for (int g = 0; g < NG; ++g) s[g] = 0.0;
  for (int c = lane; c < n3; c += 32) {
    const int yk = c % (Ak + 1), r = c / (Ak + 1), yj = r % (Aj + 1), yi = r / (Aj + 1);
    const double cijk = cp2c_at(v, ni, li, yi) * cp2c_at(v, nj, lj, yj) * cp2c_at(v, nk, lk, yk);
    for (int yl = 0; yl <= Al; ++yl) {
      const int e = ((yi + yj - yk - yl) % 4 + 4) % 4;
      if (!(e & 1)) continue;
      const double w = (e == 1 ? cijk : -cijk) * cp2c_at(v, nl, ll, yl);
      const double* x = X + idx4(n1, Ai - yi, Aj - yj, Ak - yk, Al - yl) * NG;
      const double* y = Y + idx4(n1, yi, yj, yk, yl) * NG;
      for (int g = 0; g < NG; ++g) s[g] += w * x[g] * y[g];
    }
  }
  warp_sum6(s);
}

// ddgr6 by a warp: lane 0 writes out[g]
__device__ void ddgr6_warp(const View& v, int lane, int ni, int li, int nj, int lj, int nk, int lk, int nl, int ll,
                           int di, int dj, int dip, double* out) {
  if (-li - lj + lk + ll + di + dj != 0) return;          // out stays 0
  const double r2 = 1.4142135623730951;
  const int p = dip ? 1 : 0, sm = di + dj;
  auto tab = [&](int d, int pp) {
    if (pp == 0) return d == 0 ? (int)X00 : d == 1 ? (int)X10 : (int)X20;
    if (d == 1) return pp == 1 ? (int)X11 : (int)X12;
    return pp == 1 ? (int)X01 : (int)X02;
  };
  double s[NG], sc;
  int tb;
  if (di == 0 && dj == 0) { tb = X00; sc = 1.0; }
  else if (sm == 2 || sm == -2) { tb = tab(2 - p, dip); sc = 2.0; }
  else if (sm == 1 || sm == -1) { tb = dj == 0 ? tab(1 - p, dip) : (int)X10; sc = -sm * r2; }
  else { tb = tab(2 - p, dip); sc = -1.0; }
  radx6_warp(v, lane, tb, ni, li, nj, lj, nk, lk, nl, ll, s);
  if (lane == 0)
    for (int g = 0; g < NG; ++g) out[g] = sc * s[g];
  if (sm == 0 && !(di == 0 && dj == 0) && dip) {
    radc6_imag_warp(v, lane, dip, ni, li, nj, lj, nk, lk, nl, ll, s);
    if (lane == 0)
      for (int g = 0; g < NG; ++g) out[g] += s[g];
  }
}

// jr_vec by a warp into J [NCG] (shared memory)
__device__ void jr_vec_warp(const View& v, int lane, int na, int la, int nb, int lb, int nc, int lc, int nd, int ld,
                            double* J) {
  for (int i = lane; i < NCG; i += 32) J[i] = 0.0;
  __syncwarp();
  const int K = v.K;
#define TBC_RW(piece, di, dj, dip) ddgr6_warp(v, lane, na, la, nb, lb, nc, lc, nd, ld, di, dj, dip, J + (piece) * NG)
  if (v.use_p) {
    TBC_RW(R0P, K, -1, 1); TBC_RW(R0Z, K, 0, 1); TBC_RW(R0M, K, +1, 1);
    TBC_RW(RP0, K, -1, 2); TBC_RW(RZ0, K, 0, 2); TBC_RW(RM0, K, +1, 2);
  }
  if (K == 1) {
    TBC_RW(RKP, +1, -1, 0); TBC_RW(RKZ, +1, 0, 0); TBC_RW(RKM, +1, +1, 0); TBC_RW(RPZ, 0, 0, 0);
  } else if (K == 0) {
    TBC_RW(RKP, 0, -1, 0); TBC_RW(RKZ, 0, 0, 0); TBC_RW(RKM, +1, 0, 0); TBC_RW(RPM, +1, -1, 0);
  } else {
    TBC_RW(RKP, -1, -1, 0); TBC_RW(RKZ, 0, -1, 0); TBC_RW(RKM, +1, -1, 0); TBC_RW(RZM, 0, 0, 0);
  }
#undef TBC_RW
  __syncwarp();
  if (lane < NG) {
    const int g = lane;
    if (K == 1) {
      J[RPM * NG + g] = J[RKZ * NG + g]; J[RZM * NG + g] = J[RKM * NG + g]; J[RPZ2 * NG + g] = J[RKP * NG + g];
    } else if (K == 0) {
      J[RPZ * NG + g] = J[RKP * NG + g]; J[RZM * NG + g] = J[RKM * NG + g];
    } else {
      J[RPZ * NG + g] = J[RKP * NG + g]; J[RPM * NG + g] = J[RKZ * NG + g]; J[RZM2 * NG + g] = J[RKM * NG + g];
    }
  }
  __syncwarp();
}

// stage 2: one CTA per radial group.  Phase A: the chunk's currents, one (term,
// branch, direct/exchange) per warp, the lanes splitting each Cartesian sum, into
// shared memory; phase B: one element per warp, the lanes splitting the chunk's
// (term, branch) pairs, reduced across the warp into the element's sums.
__global__ void __launch_bounds__(TBC_THREADS) k_tbc_field(View v) {
  extern __shared__ double sj[];                 // [TBC_TCH][2][2][NCG]
  __shared__ int ok[TBC_TCH][2];
  const int grp = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int e0 = v.goff[grp], e1 = v.goff[grp + 1];
  const int* q = v.gq + 4 * grp;
  const int ra = q[0], la = q[1], rc = q[2], lc = q[3];
  for (int t0 = 0; t0 < v.nt; t0 += TBC_TCH) {
    for (int it = warp; it < TBC_TCH * 4; it += nw) {
      const int tt = it >> 2, br = (it >> 1) & 1, de = it & 1, t = t0 + tt;
      int lb = 0, ld = 0, sd, sb;
      double sign;
      const bool valid = t < v.nt && term_branch(v, t, br, la, lc, &lb, &ld, &sd, &sb, &sign);
      if (lane == 0 && de == 0) ok[tt][br] = valid ? 1 : 0;
      if (!valid) continue;
      const int rb = v.tq[5 * t + 3], rd = v.tq[5 * t + 4];
      double* J = sj + (size_t)it * NCG;
      if (de == 0) jr_vec_warp(v, lane, ra, la, rb, lb, rc, lc, rd, ld, J);
      else jr_vec_warp(v, lane, ra, la, rb, lb, rd, ld, rc, lc, J);
    }
    __syncthreads();
    for (int e = e0 + warp; e < e1; e += nw) {
      double gam[6] = {0, 0, 0, 0, 0, 0};
      for (int it = lane; it < TBC_TCH * 2; it += 32) {
        const int tt = it >> 1, br = it & 1;
        if (ok[tt][br]) {
          const double* jd = sj + (size_t)((tt * 2 + br) * 2) * NCG;
          stage2_elem(v, grp, e, t0 + tt, br, jd, jd + NCG, gam);
        }
      }
      warp_sum6(gam);
      if (lane == 0) {
        double* a = v.acc + (size_t)e * 6;
        for (int k = 0; k < 6; ++k) a[k] += gam[k];
      }
    }
    __syncthreads();
  }
}
#endif

}  // namespace tbc
