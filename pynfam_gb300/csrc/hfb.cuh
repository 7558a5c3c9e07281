// HFB reconstruction on the GPU: the steps of rebuilding an HFBTHO ground state from
// its .hel fields that carry the arithmetic (HFBTHO re-run for zero iterations, as the
// reference does through hfbtho_interface.f90):
//
//  * k_hfb_basis      oscillator basis functions and their derivatives on the
//                     Gauss-Hermite x Gauss-Laguerre mesh, quadrature weights mixed
//                     in (gaupol, hfbtho_solver.f90:3463-3671; optHFBTHO :4237-4314)
//  * k_hfb_matrices   the HFB matrix (h, Delta) of every Omega block from the mean and
//                     pairing fields: every element a mesh sum of weighted products of
//                     two basis functions (gamdel, hfbtho_solver.f90:5190-5302)
//  * k_jacobi         the per-block eigensolve of [[h - lambda, Delta], [Delta,
//                     -h + lambda]] (hfbdiag's DSYEVR, hfbtho_solver.f90:1441-1972):
//                     a batched cyclic Jacobi, one CTA per matrix, parallel
//                     (round-robin) rotation order
//  * k_hfb_densities  rho, tau and the Laplacian of rho on the mesh from the final
//                     quasiparticles (DENSIT, hfbtho_solver.f90:4318-4734)
//
// The particle-number loop around the eigensolves (ALambda) and the bookkeeping stay
// on the host.  Per-item arithmetic is in __host__ __device__ functions (HFB_HD).
#pragma once

#include <cmath>
#include <cstddef>

#ifdef __CUDACC__
#define HFB_HD __host__ __device__
#else
#define HFB_HD
#endif

namespace hfbk {

// ---------------------------------------------------------------------------------
// basis functions: one (state, mesh point) item
// ---------------------------------------------------------------------------------
struct BasisView {
  int ngh, ngl, nt;
  const double *xh, *wh, *xl, *wl;
  double bz, bp;
  const int *nr, *nz, *nl;
  double* out;     // [4][nt][ngh*ngl]: function, d/dr, d/dz, (r, z) Laplacian part
};

HFB_HD inline void basis_item(const BasisView& b, int t, int r) {
  const int nghl = b.ngh * b.ngl;
  const int ih = r % b.ngh, il = r / b.ngh;
  const double x = b.xh[ih], w = b.wh[ih], xl = b.xl[il], wl = b.wl[il];
  const int nz = b.nz[t], nr = b.nr[t], l = b.nl[t];
  const double s2 = 1.4142135623730951;
  // Hermite functions up to nz
  const double w0 = pow(3.141592653589793, -0.25) * exp(-0.5 * x * x) * sqrt(w);
  double h0 = w0, h1 = s2 * w0 * x, d0 = -w0 * x, d1 = s2 * w0 * (1.0 - x * x);
  double hq = nz == 0 ? h0 : h1, hd = nz == 0 ? d0 : d1;
  for (int n = 2; n <= nz; ++n) {
    const double hn = (s2 * x * h1 - sqrt((double)(n - 1)) * h0) / sqrt((double)n);
    hd = sqrt(2.0 * n) * h1 - x * hn;
    h0 = h1; h1 = hn; hq = hn;
  }
  // Laguerre functions of this l up to nr
  double fl = 1.0;
  for (int k = 2; k <= l; ++k) fl *= (double)k;
  const double wfl = 1.0 / sqrt(fl);               // 1 / sqrt(l!)
  const double wfl1 = 1.0 / sqrt(fl * (l + 1));    // 1 / sqrt((l+1)!)
  const double w00 = s2 * exp(-0.5 * xl);
  const double wq = w00 * sqrt(0.5 * wl * pow(xl, (double)l));
  double l0 = wfl * wq, l1 = (l + 1 - xl) * wfl1 * wq;
  double e0 = (l - xl) * wfl * wq, e1 = ((double)(l * l + l) - xl * (double)(l + l + 3) + xl * xl) * wfl1 * wq;
  double lq = nr == 0 ? l0 : l1, ld = nr == 0 ? e0 : e1;
  for (int n = 2; n <= nr; ++n) {
    const double dsq = sqrt((double)n) * sqrt((double)(n + l));
    const double c1 = (double)(n + n + l - 1) - xl;
    const double c2 = sqrt((double)(n - 1)) * sqrt((double)(n - 1 + l));
    const double c3 = (double)(n + n + l) - xl;
    const double ln = (c1 * l1 - c2 * l0) / dsq;
    ld = c3 * ln - 2.0 * dsq * l1;
    l0 = l1; l1 = ln; lq = ln;
  }
  const double v2 = 0.5 / xl, v4 = v2 * v2;
  const double q = hq * lq;
  const size_t o = (size_t)t * nghl + r, plane = (size_t)b.nt * nghl;
  b.out[o] = q;
  b.out[plane + o] = (2.0 * sqrt(xl) / b.bp) * (hq * ld * v2);
  b.out[2 * plane + o] = hd * lq / b.bz;
  const double cz = nz + nz + 1, cr = nr + nr + l + 1;
  b.out[3 * plane + o] = ((x * x - cz) / (b.bz * b.bz) + 4.0 * (0.25 - cr * v2 + (double)l * l * v4) * xl / (b.bp * b.bp)) * q;
}

// ---------------------------------------------------------------------------------
// HFB matrix: one (isospin, block, i >= j) item
// ---------------------------------------------------------------------------------
enum { F_V, F_VHB, F_VR, F_VZ, F_VD, F_VS, F_VSFIZ, F_VSZFI, F_VSFIR, F_VSRFI, F_DV, NFIELD };

struct MatView {
  int nb, nt, nghl;
  const int* bstart;     // [nb+1] first state of each block
  const int* ns;         // [nt]
  const double* basis;   // [4][nt][nghl]
  const double* y;       // [nghl] 1/r
  const double* xlam;    // [nb] Lambda of spin-up states
  const double* xlap;    // [nb] Lambda of spin-down states
  const double* fields;  // [2][NFIELD][nghl]
  const size_t* moff;    // [2 * nb] start of (isospin, block) in out; h then Delta, nd*nd each
  double* out;
};

HFB_HD inline void matrix_item(const MatView& m, int it, int ib, int i, int j) {
  const int s0 = m.bstart[ib], nd = m.bstart[ib + 1] - s0;
  const int a = s0 + i, b = s0 + j;
  const size_t plane = (size_t)m.nt * m.nghl;
  const double *qa = m.basis + (size_t)a * m.nghl, *qb = m.basis + (size_t)b * m.nghl;
  const double *ra = qa + plane, *rb = qb + plane, *za = qa + 2 * plane, *zb = qb + 2 * plane;
  const double *da = qa + 3 * plane, *dbb = qb + 3 * plane;
  const double* f = m.fields + (size_t)it * NFIELD * m.nghl;
  const double *v = f + F_V * m.nghl, *vd = f + F_VD * m.nghl, *vhb = f + F_VHB * m.nghl, *vs = f + F_VS * m.nghl;
  const double *vr = f + F_VR * m.nghl, *vz = f + F_VZ * m.nghl, *vsfiz = f + F_VSFIZ * m.nghl;
  const double *vszfi = f + F_VSZFI * m.nghl, *vsfir = f + F_VSFIR * m.nghl, *vsrfi = f + F_VSRFI * m.nghl;
  const double* dv = f + F_DV * m.nghl;
  const double lam = m.xlam[ib], lap = m.xlap[ib];
  const bool ua = m.ns[a] > 0, ub = m.ns[b] > 0;
  double h = 0.0, dl = 0.0;
  for (int r = 0; r < m.nghl; ++r) {
    const double y = m.y[r];
    const double w2 = 2.0 * vd[r] + vhb[r];
    if (ua == ub) {
      // same spin: Lambda = Omega -/+ 1/2 for up/down
      const double L = ua ? lam : lap, sg = ua ? 1.0 : -1.0;
      const double Ly = L * y, Ly2 = L * L * y * y;
      const double d2a = da[r] - Ly2 * qa[r], d2b = dbb[r] - Ly2 * qb[r];
      h += qa[r] * qb[r] * (v[r] + sg * 2.0 * Ly * vsfiz[r] + Ly2 * w2) + ra[r] * rb[r] * w2 + za[r] * zb[r] * w2 +
           vd[r] * (qa[r] * d2b + d2a * qb[r]) + (vr[r] + sg * Ly * vs[r]) * (ra[r] * qb[r] + qa[r] * rb[r]) +
           vz[r] * (za[r] * qb[r] + qa[r] * zb[r]);
      dl += qa[r] * qb[r] * dv[r];
    } else {
      const double lamy = lam * y, lapy = lap * y, lampy = lamy + lapy;
      if (!ua) {   // a down, b up
        h += -ra[r] * vs[r] * zb[r] + za[r] * vs[r] * rb[r] + za[r] * (-lamy * vs[r] - vszfi[r]) * qb[r] +
             qa[r] * (-lapy * vs[r] + vszfi[r]) * zb[r] - ra[r] * vsrfi[r] * qb[r] + qa[r] * vsrfi[r] * rb[r] +
             qa[r] * lampy * vsfir[r] * qb[r];
      } else {     // a up, b down
        h += ra[r] * vs[r] * zb[r] - za[r] * vs[r] * rb[r] + za[r] * (-lapy * vs[r] + vszfi[r]) * qb[r] +
             qa[r] * (-lamy * vs[r] - vszfi[r]) * zb[r] + ra[r] * vsrfi[r] * qb[r] - qa[r] * vsrfi[r] * rb[r] +
             qa[r] * lampy * vsfir[r] * qb[r];
      }
    }
  }
  // the reference computes (n1, n2 <= n1) and uses it for both
  double* H = m.out + m.moff[2 * (size_t)ib + it];
  double* D = H + (size_t)nd * nd;
  H[(size_t)i * nd + j] = h; H[(size_t)j * nd + i] = h;
  D[(size_t)i * nd + j] = dl; D[(size_t)j * nd + i] = dl;
}

// ---------------------------------------------------------------------------------
// batched symmetric eigensolver: cyclic Jacobi in round-robin order
// ---------------------------------------------------------------------------------
// pair k of round r among m (even) indices: index m-1 is fixed, the others rotate
HFB_HD inline void rr_pair(int r, int k, int m, int* p, int* q) {
  int a, b;
  if (k == 0) { a = m - 1; b = r; }
  else { a = (r + k) % (m - 1); b = (r - k + (m - 1)) % (m - 1); }
  *p = a < b ? a : b;
  *q = a < b ? b : a;
}

// rotation (c, s) that zeroes A[p][q] in J^T A J, J = [[c, s], [-s, c]] on (p, q)
// (the symmetric Schur decomposition of Golub & Van Loan, Alg. 8.4.1)
HFB_HD inline void jacobi_cs(double app, double aqq, double apq, double* c, double* s) {
  if (apq == 0.0) { *c = 1.0; *s = 0.0; return; }
  const double tau = (aqq - app) / (2.0 * apq);
  const double t = tau >= 0.0 ? 1.0 / (tau + sqrt(1.0 + tau * tau)) : -1.0 / (-tau + sqrt(1.0 + tau * tau));
  *c = 1.0 / sqrt(1.0 + t * t);
  *s = t * (*c);
}

// row step of a round: rows p and q of A for column j
HFB_HD inline void jacobi_row(double* A, int n, int p, int q, double c, double s, int j) {
  const double ap = A[(size_t)p * n + j], aq = A[(size_t)q * n + j];
  A[(size_t)p * n + j] = c * ap - s * aq;
  A[(size_t)q * n + j] = s * ap + c * aq;
}

// column step of a round: columns p and q of A for row i
HFB_HD inline void jacobi_col(double* A, int n, int p, int q, double c, double s, int i) {
  const double ap = A[(size_t)i * n + p], aq = A[(size_t)i * n + q];
  A[(size_t)i * n + p] = c * ap - s * aq;
  A[(size_t)i * n + q] = s * ap + c * aq;
}

// the same rotation of the eigenvectors, kept transposed (VT[c][i] = V[i][c]: the
// rotated columns p and q are contiguous rows of VT)
HFB_HD inline void jacobi_vt(double* VT, int n, int p, int q, double c, double s, int i) {
  const double vp = VT[(size_t)p * n + i], vq = VT[(size_t)q * n + i];
  VT[(size_t)p * n + i] = c * vp - s * vq;
  VT[(size_t)q * n + i] = s * vp + c * vq;
}

HFB_HD inline void jacobi_zero(double* A, int n, int p, int q) {
  A[(size_t)p * n + q] = 0.0;
  A[(size_t)q * n + p] = 0.0;
}

constexpr int JAC_MAX_SWEEPS = 60;
constexpr double JAC_TOL = 1e-15;   // off-diagonal Frobenius norm / Frobenius norm at convergence

#ifdef __CUDACC__
constexpr int JAC_THREADS = 1024;
constexpr int JAC_MAXN = 512;
constexpr int JAC_SMEM_N = 164;     // matrices up to this size are rotated in shared memory (+8 KB static)

__global__ void k_hfb_basis(BasisView b) {
  const long long total = (long long)b.nt * b.ngh * b.ngl;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x)
    basis_item(b, (int)(i / (b.ngh * b.ngl)), (int)(i % (b.ngh * b.ngl)));
}

// items: (isospin, block, i >= j), enumerated by the host in `items` [n][4]
__global__ void k_hfb_matrices(MatView m, const int* items, int nitems) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nitems; i += gridDim.x * blockDim.x)
    matrix_item(m, items[4 * i], items[4 * i + 1], items[4 * i + 2], items[4 * i + 3]);
}

// one CTA per matrix: A (row-major; its diagonal ends as the eigenvalues), V <- the
// eigenvectors, transposed (row c of V holds eigenvector c); status[mat] = sweeps
// used, or -1 if not converged.
// V0 (optional): starting vectors (the previous eigenvectors of a matrix that has
// changed a little): the rotations start from V0^T A V0 with V = V0.  smem_n > 0: the
// matrices (all of size <= smem_n) are worked on in dynamic shared memory.
__global__ void __launch_bounds__(JAC_THREADS) k_jacobi(double* A, double* V, const double* V0, const long long* off,
                                                       const int* dim, int* status, int smem_n) {
  extern __shared__ double sA[];
  __shared__ double cs_c[JAC_MAXN / 2], cs_s[JAC_MAXN / 2];
  __shared__ int pp[JAC_MAXN / 2], qq[JAC_MAXN / 2];
  __shared__ double red[JAC_THREADS];
  __shared__ double s_norm;
  __shared__ int s_done;
  const int mat = blockIdx.x, n = dim[mat];
  double* ag = A + off[mat];
  double* a = smem_n > 0 ? sA : ag;
  double* v = V + off[mat];
  const int m = n + (n & 1);
  if (smem_n > 0)
    for (int i = threadIdx.x; i < n * n; i += blockDim.x) a[i] = ag[i];
  __syncthreads();
  if (V0) {
    const double* v0 = V0 + off[mat];
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {      // T = A V0 (in V)
      const int i = idx / n, j = idx % n;
      double t = 0.0;
      for (int k = 0; k < n; ++k) t += a[(size_t)i * n + k] * v0[(size_t)k * n + j];
      v[idx] = t;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {      // A = V0^T T
      const int i = idx / n, j = idx % n;
      double t = 0.0;
      for (int k = 0; k < n; ++k) t += v0[(size_t)k * n + i] * v[(size_t)k * n + j];
      a[idx] = t;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
      const int i = idx / n, j = idx % n;
      if (i < j) {
        const double x = 0.5 * (a[(size_t)i * n + j] + a[(size_t)j * n + i]);
        a[(size_t)i * n + j] = x;
        a[(size_t)j * n + i] = x;
      }
    }
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {   // VT = V0^T
      const int c = idx / n, i = idx % n;
      v[idx] = v0[(size_t)i * n + c];
    }
  } else {
    for (int i = threadIdx.x; i < n * n; i += blockDim.x) v[i] = (i / n == i % n) ? 1.0 : 0.0;
  }
  __syncthreads();
  // Frobenius norm of A (unchanged by the rotations)
  double s = 0.0;
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) s += a[i] * a[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) { s_norm = sqrt(red[0]); s_done = 0; }
  __syncthreads();
  int sweep = 0;
  for (; sweep < JAC_MAX_SWEEPS && n > 1; ++sweep) {
    // convergence: off-diagonal norm
    double o = 0.0;
    for (int i = threadIdx.x; i < n * n; i += blockDim.x)
      if (i / n != i % n) o += a[i] * a[i];
    red[threadIdx.x] = o;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) s_done = sqrt(red[0]) <= JAC_TOL * s_norm ? 1 : 0;
    __syncthreads();
    if (s_done) break;
    for (int r = 0; r < m - 1; ++r) {
      for (int k = threadIdx.x; k < m / 2; k += blockDim.x) {
        int p, q;
        rr_pair(r, k, m, &p, &q);
        double c = 1.0, sn = 0.0;
        if (q < n) jacobi_cs(a[(size_t)p * n + p], a[(size_t)q * n + q], a[(size_t)p * n + q], &c, &sn);
        pp[k] = p; qq[k] = q < n ? q : -1; cs_c[k] = c; cs_s[k] = sn;
      }
      __syncthreads();
#pragma unroll 4
      for (int it = threadIdx.x; it < (m / 2) * n; it += blockDim.x) {
        const int k = it / n, j = it % n;
        if (qq[k] >= 0 && cs_s[k] != 0.0) jacobi_row(a, n, pp[k], qq[k], cs_c[k], cs_s[k], j);
      }
      __syncthreads();
#pragma unroll 4
      for (int it = threadIdx.x; it < (m / 2) * n; it += blockDim.x) {
        const int k = it / n, i = it % n;
        if (qq[k] >= 0 && cs_s[k] != 0.0) {
          jacobi_col(a, n, pp[k], qq[k], cs_c[k], cs_s[k], i);
          jacobi_vt(v, n, pp[k], qq[k], cs_c[k], cs_s[k], i);
        }
      }
      __syncthreads();
      // the rotated element is zero in exact arithmetic
      for (int k = threadIdx.x; k < m / 2; k += blockDim.x)
        if (qq[k] >= 0 && cs_s[k] != 0.0) jacobi_zero(a, n, pp[k], qq[k]);
      __syncthreads();
    }
  }
  if (smem_n > 0)
    for (int i = threadIdx.x; i < n; i += blockDim.x) ag[(size_t)i * n + i] = a[(size_t)i * n + i];
  if (threadIdx.x == 0) status[mat] = (n <= 1 || s_done) ? sweep : -1;
}
#endif

// ---------------------------------------------------------------------------------
// local densities: one (block, mesh point) item, un-normalised sums of DENSIT
// ---------------------------------------------------------------------------------
struct DensView {
  int nb, nt, nghl;
  const int* bstart;
  const int* ns;
  const double* basis;   // [4][nt][nghl]
  const double* y;
  const double* xlam;
  const double* xlap;
  const size_t* woff;    // [nb] start of the block's [nd][nd] matrices
  const double* W;       // V per block, row = state, column = quasiparticle (inactive columns zero)
  const double* U;       // U per block (finite temperature) or null
  const double* f;       // [nt] thermal occupation of each quasiparticle (block order) or null
  double* out;           // [3][nghl]: rho, tau, Laplacian-of-rho sums
};

HFB_HD inline void density_item(const DensView& d, int ib, int r, double* acc) {
  const int s0 = d.bstart[ib], nd = d.bstart[ib + 1] - s0;
  const size_t plane = (size_t)d.nt * d.nghl;
  const double y2 = d.y[r] * d.y[r];
  const double xl2 = d.xlam[ib] * d.xlam[ib] * y2, xp2 = d.xlap[ib] * d.xlap[ib] * y2;
  acc[0] = acc[1] = acc[2] = 0.0;
  for (int part = 0; part < (d.U ? 2 : 1); ++part) {
    const double* M = (part == 0 ? d.W : d.U) + d.woff[ib];
    for (int k = 0; k < nd; ++k) {
      double fu = 0, fd = 0, fur = 0, fdr = 0, fuz = 0, fdz = 0, fu2 = 0, fd2 = 0;
      bool any = false;
      for (int i = 0; i < nd; ++i) {
        const double w = M[(size_t)i * nd + k];
        if (w == 0.0) continue;
        any = true;
        const size_t o = (size_t)(s0 + i) * d.nghl + r;
        const double q = d.basis[o], qr = d.basis[plane + o], qz = d.basis[2 * plane + o], q2 = d.basis[3 * plane + o];
        if (d.ns[s0 + i] > 0) { fu += w * q; fur += w * qr; fuz += w * qz; fu2 += w * q2; }
        else { fd += w * q; fdr += w * qr; fdz += w * qz; fd2 += w * q2; }
      }
      if (!any) continue;
      double wk = 1.0;
      if (d.f) wk = part == 0 ? 1.0 - d.f[s0 + k] : d.f[s0 + k];
      const double tw = fur * fur + fdr * fdr + fuz * fuz + fdz * fdz;
      acc[0] += wk * (fu * fu + fd * fd);
      acc[1] += wk * (xl2 * fu * fu + xp2 * fd * fd + tw);
      acc[2] += wk * (fu * fu2 + fd * fd2 + tw);
    }
  }
}

#ifdef __CUDACC__
__global__ void k_hfb_densities(DensView d) {
  const int total = d.nb * d.nghl;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    double acc[3];
    const int ib = i / d.nghl, r = i % d.nghl;
    density_item(d, ib, r, acc);
    for (int c = 0; c < 3; ++c) atomicAdd(d.out + (size_t)c * d.nghl + r, acc[c]);
  }
}
#endif

}  // namespace hfbk
