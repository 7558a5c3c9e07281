// Device kernels of the pnFAM solver (sm_103a).
//
// One FAM iteration (pnfam_solver.f90:114-209) for a batch of omega points:
//   k_gemm        grouped multi-term FP64 block GEMM, used for the basis
//                 changes dR_qp -> dR_sp (pnfam_solver.f90:144-150) and
//                 dH_sp -> dH_qp (:160-166), and F_sp -> F_qp (:368-381)
//   k_density     fused sum_a phi_a rho_ab + reduction over b into the 28
//                 local densities (pnfam_hamiltonian_blas.f90:124-711)
//   k_meanfield   densities -> field tensor mf(0:4,0:4,s,s') and the pairing
//                 fields (pnfam_hamiltonian_blas.f90:775-1094, 1201-1208)
//   k_hproj       h_ab = 2 sum_r phi_a (mf phi_b), Delta_ab likewise
//                 (pnfam_hamiltonian_blas.f90:1107-1167, 1212-1260)
//   k_green       dR = G o (q dH + F)  (pnfam_solver.f90:169-183, 510-544)
//   k_bro_*       modified Broyden mixing (pnfam_broyden.f90:117-216)
//   k_contract    S = -1/pi sum F dR  (pnfam_type_bbm.f90:393-421)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pnfam {

// ---------------------------------------------------------------------------
// grouped multi-term GEMM
// ---------------------------------------------------------------------------
enum BufId { B_UP = 0, B_VP, B_UN, B_VN, B_STATE, B_T, B_RSP, B_HSP, B_HQP, NBUF };

template <class T>
struct BufDescT {
  T* base;
  long long sp;   // stride between points
  long long spl;  // stride between the Re and Im planes
};
using BufDesc = BufDescT<double>;

struct GemmTerm {
  long long aoff, boff;
  int abuf, bbuf;
  int lda, ldb;
  int tA, tB;          // 0 = as stored, 1 = transposed
  double alpha[2];     // per plane (Re, Im)
};

#define PNFAM_MAXTERM 4
struct GemmTask {
  int M, N, K, nterm;
  GemmTerm t[PNFAM_MAXTERM];
  long long coff;
  int cbuf, ldc;
  int tile0, ntn;      // first tile in the flattened grid, tiles along N
};

#define GT 32
#define GK 16

template <class T>
__device__ __forceinline__ const T* bufptr(const BufDescT<T>* b, int id, int p, int plane, long long off) {
  const BufDescT<T> d = b[id];
  return d.base + (long long)p * d.sp + (long long)plane * d.spl + off;
}

// C = sum_t alpha_t op(A_t) op(B_t); blockIdx.y = point*2 + plane; T = compute type
template <class T>
__global__ void __launch_bounds__(256) k_gemm(const GemmTask* __restrict__ tasks, const int* __restrict__ tile2task,
                                              const BufDescT<T>* __restrict__ bufs, const int* __restrict__ active) {
  const int z = blockIdx.y;
  const int p = z >> 1, plane = z & 1;
  if (active && !active[p]) return;
  const int tile = blockIdx.x;
  const GemmTask& Tk = tasks[tile2task[tile]];
  const int lt = tile - Tk.tile0;
  const int m0 = (lt / Tk.ntn) * GT, n0 = (lt % Tk.ntn) * GT;
  __shared__ T As[GK][GT + 1];
  __shared__ T Bs[GK][GT + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  T acc00 = 0, acc01 = 0, acc10 = 0, acc11 = 0;
  const int M = Tk.M, N = Tk.N, K = Tk.K;
  for (int it = 0; it < Tk.nterm; ++it) {
    const GemmTerm& tm = Tk.t[it];
    const T* A = bufptr(bufs, tm.abuf, p, plane, tm.aoff);
    const T* B = bufptr(bufs, tm.bbuf, p, plane, tm.boff);
    const T alpha = (T)tm.alpha[plane];
    for (int k0 = 0; k0 < K; k0 += GK) {
      for (int e = threadIdx.x; e < GK * GT; e += 256) {
        const int kk = e / GT, mm = e % GT;
        const int gm = m0 + mm, gk = k0 + kk;
        T v = 0;
        if (gm < M && gk < K) v = tm.tA ? A[gk + (long long)gm * tm.lda] : A[gm + (long long)gk * tm.lda];
        As[kk][mm] = alpha * v;
        const int gn = n0 + mm;
        T w = 0;
        if (gn < N && gk < K) w = tm.tB ? B[gn + (long long)gk * tm.ldb] : B[gk + (long long)gn * tm.ldb];
        Bs[kk][mm] = w;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < GK; ++kk) {
        const T a0 = As[kk][ty * 2], a1 = As[kk][ty * 2 + 1];
        const T b0 = Bs[kk][tx * 2], b1 = Bs[kk][tx * 2 + 1];
        acc00 = fma(a0, b0, acc00); acc01 = fma(a0, b1, acc01);
        acc10 = fma(a1, b0, acc10); acc11 = fma(a1, b1, acc11);
      }
      __syncthreads();
    }
  }
  T* C = const_cast<T*>(bufptr(bufs, Tk.cbuf, p, plane, Tk.coff));
  const int r0 = m0 + ty * 2, c0 = n0 + tx * 2;
  if (r0 < M && c0 < N) C[r0 + (long long)c0 * Tk.ldc] = acc00;
  if (r0 < M && c0 + 1 < N) C[r0 + (long long)(c0 + 1) * Tk.ldc] = acc01;
  if (r0 + 1 < M && c0 < N) C[r0 + 1 + (long long)c0 * Tk.ldc] = acc10;
  if (r0 + 1 < M && c0 + 1 < N) C[r0 + 1 + (long long)(c0 + 1) * Tk.ldc] = acc11;
}

// ---------------------------------------------------------------------------
// basis on device
// ---------------------------------------------------------------------------
template <class T>
struct DevBasisT {
  int nb, dqp, nghl;
  const int* db;
  const int* st;
  const int* nup;
  const signed char* ns;
  const T* phi;          // [5][dqp][nghl]
  const double* wdcori;
  const double* crho;
  const double* cs;
  const double* cpair;
  const double* cspair;
  double sc[12];         // cdrho, ctau, ctj0, ctj1, ctj2, crdj, cds, ct, cj, cgs, cf, csdj
};
using DevBasis = DevBasisT<double>;

enum { ND = 28 };  // complex local densities
// 0 rho 1 tau 2 tjrr 3 tjpr 4 tjzr 5 tjrp 6 tjpp 7 tjzp 8 tjrz 9 tjpz 10 tjzz
// 11 sr 12 sp 13 sz 14 tr 15 tp 16 tz 17 jr 18 jp 19 jz 20 fr 21 fp 22 fz 23 gs
// 24 rb 25 sbr 26 sbp 27 sbz
enum { D_RHO = 0, D_TAU, D_TJRR, D_TJPR, D_TJZR, D_TJRP, D_TJPP, D_TJZP, D_TJRZ, D_TJPZ, D_TJZZ,
       D_SR, D_SP, D_SZ, D_TR, D_TP, D_TZ, D_JR, D_JP, D_JZ, D_FR, D_FP, D_FZ, D_GS,
       D_RB, D_SBR, D_SBP, D_SBZ };

// One density call: rho in structure (rcols, roffs), kappa in (kcols, koffs), both
// [P][2 planes][plane stride] at the given base/offset.
template <class T>
struct DensCallT {
  const T* rho; long long rho_sp, rho_spl;
  const int* rcols; const long long* roffs;
  const T* kap; long long kap_sp, kap_spl;
  const int* kcols; const long long* koffs;
};
using DensCall = DensCallT<double>;

#define DRT 32   // mesh points per CTA
#define DBC 8    // b columns per chunk
#define DAK 16   // a rows per chunk

template <class T>
__device__ __forceinline__ T red8(T v) {
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  return v;
}

// grid (ceil(nghl/DRT), G, P*2 calls); block 256 = DRT r x DBC b
// dpart: [P][2][G][2*ND][nghl]
template <class T>
__global__ void __launch_bounds__(256) k_density(DevBasisT<T> B, DensCallT<T> c0, DensCallT<T> c1, int G,
                                                 T* __restrict__ dpart, const int* __restrict__ active) {
  const int p = blockIdx.z >> 1, call = blockIdx.z & 1;
  if (!active[p]) return;
  const DensCallT<T>& C = call ? c1 : c0;
  const int g = blockIdx.y;
  const int r0 = blockIdx.x * DRT;
  const int rl = threadIdx.x >> 3, bl = threadIdx.x & 7;
  const int nghl = B.nghl;
  const int r = r0 + rl;
  const bool rok = r < nghl;
  __shared__ T acc[2 * ND][DRT];
  __shared__ T sphi[4][DAK][DRT];
  __shared__ T srho[2][DAK][DBC];
  for (int e = threadIdx.x; e < 2 * ND * DRT; e += 256) (&acc[0][0])[e] = 0;
  __syncthreads();
  const long long ps = (long long)B.dqp * nghl;
  const T h5 = (T)0.5, two = (T)2;

#define ACC(k, re, im)                                   \
  {                                                      \
    const T vr_ = red8<T>(re), vi_ = red8<T>(im);       \
    if (bl == 0) { acc[2 * (k)][rl] += vr_; acc[2 * (k) + 1][rl] += vi_; } \
  }

  // ---------------- normal densities ----------------
  for (int ix = g; ix < B.nb; ix += G) {
    const int iy = C.rcols[ix];
    if (iy < 0) continue;
    const int d = B.db[ix], dc = B.db[iy], nu = B.nup[ix];
    const int sa = B.st[ix], sb = B.st[iy];
    const T* rho = C.rho + (long long)p * C.rho_sp + C.roffs[ix];
    for (int b0 = 0; b0 < dc; b0 += DBC) {
      const int b = b0 + bl;
      T w[2][4][2];
#pragma unroll
      for (int s = 0; s < 2; ++s)
#pragma unroll
        for (int q = 0; q < 4; ++q) { w[s][q][0] = 0; w[s][q][1] = 0; }
      for (int a0 = 0; a0 < d; a0 += DAK) {
        const int na = min(DAK, d - a0);
        for (int e = threadIdx.x; e < 4 * DAK * DRT; e += 256) {
          const int q = e / (DAK * DRT), rem = e % (DAK * DRT), aa = rem / DRT, rr = rem % DRT;
          T v = 0;
          if (aa < na && r0 + rr < nghl) v = B.phi[q * ps + (long long)(sa + a0 + aa) * nghl + r0 + rr];
          sphi[q][aa][rr] = v;
        }
        for (int e = threadIdx.x; e < 2 * DAK * DBC; e += 256) {
          const int pl = e / (DAK * DBC), rem = e % (DAK * DBC), aa = rem / DBC, bb = rem % DBC;
          T v = 0;
          if (aa < na && b0 + bb < dc) v = rho[(long long)pl * C.rho_spl + (a0 + aa) + (long long)(b0 + bb) * d];
          srho[pl][aa][bb] = v;
        }
        __syncthreads();
        // spin-up rows first: split the chunk at the spin boundary
        const int nup_here = max(0, min(na, nu - a0));
        for (int aa = 0; aa < nup_here; ++aa) {
          const T re = srho[0][aa][bl], im = srho[1][aa][bl];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const T f = sphi[q][aa][rl];
            w[0][q][0] = fma(f, re, w[0][q][0]); w[0][q][1] = fma(f, im, w[0][q][1]);
          }
        }
        for (int aa = nup_here; aa < na; ++aa) {
          const T re = srho[0][aa][bl], im = srho[1][aa][bl];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const T f = sphi[q][aa][rl];
            w[1][q][0] = fma(f, re, w[1][q][0]); w[1][q][1] = fma(f, im, w[1][q][1]);
          }
        }
        __syncthreads();
      }
      // epilogue: contributions of column b at mesh point r
      T P0 = 0, P1 = 0, P2 = 0, P3 = 0, sg = 0;
      const bool ok = rok && b < dc;
      if (ok) {
        const int jb = sb + b;
        P0 = B.phi[0 * ps + (long long)jb * nghl + r];
        P1 = B.phi[1 * ps + (long long)jb * nghl + r];
        P2 = B.phi[2 * ps + (long long)jb * nghl + r];
        P3 = B.phi[3 * ps + (long long)jb * nghl + r];
        sg = (T)B.ns[jb];
      }
      const int si = (sg > 0) ? 0 : 1;  // same-spin set of wfa
      // select S (same spin as b) and O (opposite)
      T Sr[4], Si[4], Or[4], Oi[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        Sr[q] = si == 0 ? w[0][q][0] : w[1][q][0]; Si[q] = si == 0 ? w[0][q][1] : w[1][q][1];
        Or[q] = si == 0 ? w[1][q][0] : w[0][q][0]; Oi[q] = si == 0 ? w[1][q][1] : w[0][q][1];
        if (!ok) { Sr[q] = Si[q] = Or[q] = Oi[q] = 0; }
      }
      const T sig = (sg < 0) ? (T)1 : (T)-1;  // +1 if b is spin down
      T xr, xi;
      // diagonal in spin
      xr = Sr[0] * P0; xi = Si[0] * P0;
      ACC(D_RHO, xr, xi);
      ACC(D_SZ, sg * xr, sg * xi);
      xr = h5 * (Sr[0] * P2 + Sr[2] * P0); xi = h5 * (Si[0] * P2 + Si[2] * P0);
      ACC(D_JP, xr, xi);
      ACC(D_TJPZ, sg * xr, sg * xi);
      xr = Sr[1] * P1 + Sr[2] * P2 + Sr[3] * P3; xi = Si[1] * P1 + Si[2] * P2 + Si[3] * P3;
      ACC(D_TAU, xr, xi);
      ACC(D_TZ, sg * xr, sg * xi);
      xr = h5 * (Sr[0] * P1 - Sr[1] * P0); xi = h5 * (Si[0] * P1 - Si[1] * P0);
      ACC(D_JR, -xi, xr);
      ACC(D_TJRZ, -sg * xi, sg * xr);
      xr = h5 * (Sr[0] * P3 - Sr[3] * P0); xi = h5 * (Si[0] * P3 - Si[3] * P0);
      ACC(D_JZ, -xi, xr);
      ACC(D_TJZZ, -sg * xi, sg * xr);
      // gs: diagonal part + off-diagonal parts
      {
        T gr = sg * (Sr[0] * P3 + Sr[3] * P0), gi = sg * (Si[0] * P3 + Si[3] * P0);
        gr += sig * (Or[0] * P2 - Or[2] * P0) + (Or[0] * P1 + Or[1] * P0);
        gi += sig * (Oi[0] * P2 - Oi[2] * P0) + (Oi[0] * P1 + Oi[1] * P0);
        ACC(D_GS, gr, gi);
      }
      {
                T fr = h5 * sg * (Sr[1] * P3 + Sr[3] * P1), fi = h5 * sg * (Si[1] * P3 + Si[3] * P1);
        fr += Or[1] * P1 + sig * h5 * (Or[1] * P2 - Or[2] * P1);
        fi += Oi[1] * P1 + sig * h5 * (Oi[1] * P2 - Oi[2] * P1);
        ACC(D_FR, fr, fi);
      }
      {
        // fp += i*sg*(S2P3 - S3P2)/2 + i*(sig*O2P2 + (O2P1 - O1P2)/2)
                const T ar = h5 * sg * (Sr[2] * P3 - Sr[3] * P2) + sig * Or[2] * P2 + h5 * (Or[2] * P1 - Or[1] * P2);
        const T ai = h5 * sg * (Si[2] * P3 - Si[3] * P2) + sig * Oi[2] * P2 + h5 * (Oi[2] * P1 - Oi[1] * P2);
        ACC(D_FP, -ai, ar);
      }
      {
                T zr = sg * Sr[3] * P3, zi = sg * Si[3] * P3;
        zr += h5 * (Or[3] * P1 + sig * Or[3] * P2 + Or[1] * P3 - sig * Or[2] * P3);
        zi += h5 * (Oi[3] * P1 + sig * Oi[3] * P2 + Oi[1] * P3 - sig * Oi[2] * P3);
        ACC(D_FZ, zr, zi);
      }
      // not diagonal in spin
      xr = Or[0] * P0; xi = Oi[0] * P0;
      ACC(D_SR, xr, xi);
      ACC(D_SP, -sig * xi, sig * xr);
      xr = h5 * (Or[2] * P0 + Or[0] * P2); xi = h5 * (Oi[2] * P0 + Oi[0] * P2);
      ACC(D_TJPR, xr, xi);
      ACC(D_TJPP, -sig * xi, sig * xr);
      xr = Or[1] * P1 + Or[2] * P2 + Or[3] * P3; xi = Oi[1] * P1 + Oi[2] * P2 + Oi[3] * P3;
      ACC(D_TR, xr, xi);
      ACC(D_TP, -sig * xi, sig * xr);
      xr = h5 * (Or[0] * P1 - Or[1] * P0); xi = h5 * (Oi[0] * P1 - Oi[1] * P0);
      ACC(D_TJRR, -xi, xr);
      ACC(D_TJRP, -sig * xr, -sig * xi);
      xr = h5 * (Or[0] * P3 - Or[3] * P0); xi = h5 * (Oi[0] * P3 - Oi[3] * P0);
      ACC(D_TJZR, -xi, xr);
      ACC(D_TJZP, -sig * xr, -sig * xi);
    }
  }
  // ---------------- pairing densities ----------------
  for (int ix = g; ix < B.nb; ix += G) {
    const int iy = C.kcols[ix];
    if (iy < 0) continue;
    const int d = B.db[ix], dc = B.db[iy], nu = B.nup[ix];
    const int sa = B.st[ix], sb = B.st[iy];
    const T* kap = C.kap + (long long)p * C.kap_sp + C.koffs[ix];
    for (int b0 = 0; b0 < dc; b0 += DBC) {
      const int b = b0 + bl;
      T w[2][2] = {{0, 0}, {0, 0}};
      for (int a0 = 0; a0 < d; a0 += DAK) {
        const int na = min(DAK, d - a0);
        for (int e = threadIdx.x; e < DAK * DRT; e += 256) {
          const int aa = e / DRT, rr = e % DRT;
          T v = 0;
          if (aa < na && r0 + rr < nghl) v = B.phi[(long long)(sa + a0 + aa) * nghl + r0 + rr];
          sphi[0][aa][rr] = v;
        }
        for (int e = threadIdx.x; e < 2 * DAK * DBC; e += 256) {
          const int pl = e / (DAK * DBC), rem = e % (DAK * DBC), aa = rem / DBC, bb = rem % DBC;
          T v = 0;
          if (aa < na && b0 + bb < dc) v = kap[(long long)pl * C.kap_spl + (a0 + aa) + (long long)(b0 + bb) * d];
          srho[pl][aa][bb] = v;
        }
        __syncthreads();
        const int nup_here = max(0, min(na, nu - a0));
        for (int aa = 0; aa < nup_here; ++aa) {
          const T f = sphi[0][aa][rl];
          w[0][0] = fma(f, srho[0][aa][bl], w[0][0]); w[0][1] = fma(f, srho[1][aa][bl], w[0][1]);
        }
        for (int aa = nup_here; aa < na; ++aa) {
          const T f = sphi[0][aa][rl];
          w[1][0] = fma(f, srho[0][aa][bl], w[1][0]); w[1][1] = fma(f, srho[1][aa][bl], w[1][1]);
        }
        __syncthreads();
      }
      T P0 = 0, sg = 0;
      const bool ok = rok && b < dc;
      if (ok) {
        const int jb = sb + b;
        P0 = B.phi[(long long)jb * nghl + r];
        sg = (T)B.ns[jb];
      }
      const int si = (sg > 0) ? 0 : 1;
      T Sr = si == 0 ? w[0][0] : w[1][0], Si = si == 0 ? w[0][1] : w[1][1];
      T Or = si == 0 ? w[1][0] : w[0][0], Oi = si == 0 ? w[1][1] : w[0][1];
      if (!ok) { Sr = Si = Or = Oi = 0; }
      const T sig = (sg < 0) ? (T)1 : (T)-1;
      T xr = two * Or * P0, xi = two * Oi * P0;
      ACC(D_RB, -sg * xr, -sg * xi);
      ACC(D_SBZ, xr, xi);
      xr = two * Sr * P0; xi = two * Si * P0;
      ACC(D_SBR, sig * xr, sig * xi);
      ACC(D_SBP, xi, -xr);
    }
  }
#undef ACC
  __syncthreads();
  T* out = dpart + (((long long)p * 2 + call) * G + g) * (2 * ND) * nghl;
  for (int e = threadIdx.x; e < 2 * ND * DRT; e += 256) {
    const int k = e / DRT, rr = e % DRT;
    if (r0 + rr < nghl) out[(long long)k * nghl + r0 + rr] = acc[k][rr];
  }
}

// ---------------------------------------------------------------------------
// mean field: mf slot (iy, iz, sa, sb) = ((iy*5 + iz)*2 + (sa<0))*2 + (sb<0);
// pairing fields at 100 + (sa<0)*2 + (sb<0)
// mf: [P][2][NMF][2][nghl]
// ---------------------------------------------------------------------------
enum { NMF = 104 };
__host__ __device__ __forceinline__ int mfslot(int iy, int iz, int sa, int sb) {
  return ((iy * 5 + iz) * 2 + (sa < 0 ? 1 : 0)) * 2 + (sb < 0 ? 1 : 0);
}

struct cplx { double r, i; };
__device__ __forceinline__ cplx cmk(double r, double i) { cplx c; c.r = r; c.i = i; return c; }
__device__ __forceinline__ cplx cadd(cplx a, cplx b) { return cmk(a.r + b.r, a.i + b.i); }
__device__ __forceinline__ cplx csc(double s, cplx a) { return cmk(s * a.r, s * a.i); }

template <class T>
__global__ void __launch_bounds__(128) k_meanfield(DevBasisT<T> B, int G, const T* __restrict__ dpart,
                                                   T* __restrict__ mfout, const int* __restrict__ active) {
  const int p = blockIdx.y >> 1, call = blockIdx.y & 1;
  if (!active[p]) return;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int nghl = B.nghl;
  if (r >= nghl) return;
  cplx d[ND];
  const T* dp = dpart + ((long long)p * 2 + call) * G * (2 * ND) * nghl;
  const double wd = B.wdcori[r];
  for (int k = 0; k < ND; ++k) {
    double sr = 0.0, si = 0.0;
    for (int g = 0; g < G; ++g) {
      sr += (double)dp[((long long)g * 2 * ND + 2 * k) * nghl + r];
      si += (double)dp[((long long)g * 2 * ND + 2 * k + 1) * nghl + r];
    }
    d[k] = cmk(sr * wd, si * wd);
  }
  const double crho = B.crho[r], cs = B.cs[r], cpair = B.cpair[r], cspair = B.cspair[r];
  const double cdrho = B.sc[0], ctau = B.sc[1], ctj0 = B.sc[2], ctj1 = B.sc[3], ctj2 = B.sc[4], crdj = B.sc[5];
  const double cds = B.sc[6], ct = B.sc[7], cj = B.sc[8], cgs = B.sc[9], cf = B.sc[10], csdj = B.sc[11];
  cplx mf[NMF];
  for (int k = 0; k < NMF; ++k) mf[k] = cmk(0.0, 0.0);
#define M_(iy, iz, sa, sb) mf[mfslot(iy, iz, sa, sb)]
#define ADD(iy, iz, sa, sb, sym, v) M_(iy, iz, sa, sb) = cadd(M_(iy, iz, sa, sb), csc(sym, v))
  const cplx rho = d[D_RHO], tau = d[D_TAU], tjrr = d[D_TJRR], tjpr = d[D_TJPR], tjzr = d[D_TJZR];
  const cplx tjrp = d[D_TJRP], tjpp = d[D_TJPP], tjzp = d[D_TJZP], tjrz = d[D_TJRZ], tjpz = d[D_TJPZ];
  const cplx tjzz = d[D_TJZZ], sr = d[D_SR], sp = d[D_SP], sz = d[D_SZ], tr = d[D_TR], tp = d[D_TP];
  const cplx tz = d[D_TZ], jr = d[D_JR], jp = d[D_JP], jz = d[D_JZ], fr = d[D_FR], fp = d[D_FP];
  const cplx fz = d[D_FZ], gs = d[D_GS];
  const cplx t0 = csc(ctj0, cadd(cadd(tjrr, tjpp), tjzz));
  const cplx t1a = csc(ctj1, cadd(tjzr, csc(-1.0, tjrz)));
  const cplx t1b = csc(ctj1, cadd(tjpz, csc(-1.0, tjzp)));
  const cplx t2a = csc(ctj2, cadd(tjrz, tjzr));
  const cplx t2b = csc(ctj2, cadd(tjpz, tjzp));
  cplx aux;
  // diagonal in spin (pnfam_hamiltonian_blas.f90:783-905)
  M_(0, 0, 1, 1) = cadd(csc(2.0 * crho, rho), csc(ctau, tau));
  M_(0, 0, -1, -1) = M_(0, 0, 1, 1);
  aux = cadd(cadd(csc(2.0 * cs, sz), csc(ct, tz)), csc(cf, fz));
  ADD(0, 0, 1, 1, 1.0, aux); ADD(0, 0, -1, -1, -1.0, aux);

  M_(0, 1, 1, 1) = csc(-crdj, cadd(tjpz, csc(-1.0, tjzp)));
  M_(0, 1, -1, -1) = M_(0, 1, 1, 1);
  aux = csc(-csdj, jp);
  ADD(0, 1, 1, 1, 1.0, aux); ADD(0, 1, -1, -1, -1.0, aux);
  M_(1, 0, 1, 1) = M_(0, 1, 1, 1);
  M_(1, 0, -1, -1) = M_(0, 1, -1, -1);
  aux = cmk(-t1a.i + 0.5 * t2a.i, t1a.r - 0.5 * t2a.r);
  ADD(0, 1, 1, 1, 1.0, aux); ADD(0, 1, -1, -1, -1.0, aux);
  ADD(1, 0, 1, 1, -1.0, aux); ADD(1, 0, -1, -1, 1.0, aux);
  aux = cmk(cj * jr.i, -cj * jr.r);
  ADD(0, 1, 1, 1, 1.0, aux); ADD(0, 1, -1, -1, 1.0, aux);
  ADD(1, 0, 1, 1, -1.0, aux); ADD(1, 0, -1, -1, -1.0, aux);

  M_(0, 2, 1, 1) = csc(cj, jp);
  M_(0, 2, -1, -1) = M_(0, 2, 1, 1);
  aux = cadd(t1b, csc(0.5, t2b));
  ADD(0, 2, 1, 1, 1.0, aux); ADD(0, 2, -1, -1, -1.0, aux);
  M_(2, 0, 1, 1) = M_(0, 2, 1, 1);
  M_(2, 0, -1, -1) = M_(0, 2, -1, -1);
  aux = cmk(-csdj * jr.i, csdj * jr.r);
  ADD(0, 2, 1, 1, 1.0, aux); ADD(0, 2, -1, -1, -1.0, aux);
  ADD(2, 0, 1, 1, -1.0, aux); ADD(2, 0, -1, -1, 1.0, aux);
  aux = cmk(crdj * (tjzr.i - tjrz.i), -crdj * (tjzr.r - tjrz.r));
  ADD(0, 2, 1, 1, 1.0, aux); ADD(0, 2, -1, -1, 1.0, aux);
  ADD(2, 0, 1, 1, -1.0, aux); ADD(2, 0, -1, -1, -1.0, aux);

  M_(0, 3, 1, 1) = csc(-crdj, cadd(tjrp, csc(-1.0, tjpr)));
  M_(0, 3, -1, -1) = M_(0, 3, 1, 1);
  aux = csc(2.0 * cgs, gs);
  ADD(0, 3, 1, 1, 1.0, aux); ADD(0, 3, -1, -1, -1.0, aux);
  M_(3, 0, 1, 1) = M_(0, 3, 1, 1);
  M_(3, 0, -1, -1) = M_(0, 3, -1, -1);
  aux = cmk(t0.i - ctj2 * (tjrr.i + tjpp.i - 2.0 * tjzz.i) / 3.0,
            -t0.r + ctj2 * (tjrr.r + tjpp.r - 2.0 * tjzz.r) / 3.0);
  ADD(0, 3, 1, 1, 1.0, aux); ADD(0, 3, -1, -1, -1.0, aux);
  ADD(3, 0, 1, 1, -1.0, aux); ADD(3, 0, -1, -1, 1.0, aux);
  aux = cmk(cj * jz.i, -cj * jz.r);
  ADD(0, 3, 1, 1, 1.0, aux); ADD(0, 3, -1, -1, 1.0, aux);
  ADD(3, 0, 1, 1, -1.0, aux); ADD(3, 0, -1, -1, -1.0, aux);

  M_(0, 4, 1, 1) = csc(2.0 * cdrho, rho);
  M_(0, 4, -1, -1) = M_(0, 4, 1, 1);
  aux = csc(2.0 * cds, sz);
  ADD(0, 4, 1, 1, 1.0, aux); ADD(0, 4, -1, -1, -1.0, aux);
  M_(4, 0, 1, 1) = M_(0, 4, 1, 1);
  M_(4, 0, -1, -1) = M_(0, 4, -1, -1);

  M_(1, 2, 1, 1) = csc(csdj, sz);
  M_(1, 2, -1, -1) = M_(1, 2, 1, 1);
  aux = csc(crdj, rho);
  ADD(1, 2, 1, 1, 1.0, aux); ADD(1, 2, -1, -1, -1.0, aux);
  M_(2, 1, 1, 1) = M_(1, 2, 1, 1);
  M_(2, 1, -1, -1) = M_(1, 2, -1, -1);

  M_(1, 3, 1, 1) = csc(0.5 * cf, sr);
  M_(1, 3, -1, -1) = csc(-1.0, M_(1, 3, 1, 1));
  M_(3, 1, 1, 1) = M_(1, 3, 1, 1);
  M_(3, 1, -1, -1) = M_(1, 3, -1, -1);
  aux = cmk(-csdj * sp.i, csdj * sp.r);
  ADD(1, 3, 1, 1, 1.0, aux); ADD(1, 3, -1, -1, 1.0, aux);
  ADD(3, 1, 1, 1, -1.0, aux); ADD(3, 1, -1, -1, -1.0, aux);

  M_(2, 3, 1, 1) = csc(-csdj, sr);
  M_(2, 3, -1, -1) = M_(2, 3, 1, 1);
  aux = cmk(0.5 * cf * sp.i, -0.5 * cf * sp.r);
  ADD(2, 3, 1, 1, 1.0, aux); ADD(2, 3, -1, -1, -1.0, aux);
  M_(3, 2, 1, 1) = M_(2, 3, -1, -1);
  M_(3, 2, -1, -1) = M_(2, 3, 1, 1);

  M_(1, 1, 1, 1) = csc(4.0 * cdrho + ctau, rho);
  M_(1, 1, -1, -1) = M_(1, 1, 1, 1);
  aux = csc(4.0 * cds + ct, sz);
  ADD(1, 1, 1, 1, 1.0, aux); ADD(1, 1, -1, -1, -1.0, aux);
  M_(2, 2, 1, 1) = M_(1, 1, 1, 1);
  M_(2, 2, -1, -1) = M_(1, 1, -1, -1);
  M_(3, 3, 1, 1) = M_(1, 1, 1, 1);
  M_(3, 3, -1, -1) = M_(1, 1, -1, -1);
  aux = csc(cf, sz);
  ADD(3, 3, 1, 1, 1.0, aux); ADD(3, 3, -1, -1, -1.0, aux);

  // not diagonal in spin (pnfam_hamiltonian_blas.f90:908-1094)
  M_(0, 0, 1, -1) = cadd(cadd(csc(2.0 * cs, sr), csc(ct, tr)), csc(cf, fr));
  M_(0, 0, -1, 1) = M_(0, 0, 1, -1);
  aux = cmk(2.0 * cs * sp.i + ct * tp.i + cf * fp.i, -2.0 * cs * sp.r - ct * tp.r - cf * fp.r);
  ADD(0, 0, 1, -1, 1.0, aux); ADD(0, 0, -1, 1, -1.0, aux);

  M_(0, 1, 1, -1) = csc(2.0 * cgs, gs);
  M_(0, 1, -1, 1) = M_(0, 1, 1, -1);
  aux = cmk(csdj * jz.i, -csdj * jz.r);
  ADD(0, 1, 1, -1, 1.0, aux); ADD(0, 1, -1, 1, -1.0, aux);
  M_(1, 0, 1, -1) = M_(0, 1, 1, -1);
  M_(1, 0, -1, 1) = M_(0, 1, -1, 1);
  M_(0, 2, 1, -1) = M_(0, 1, 1, -1);
  M_(2, 0, -1, 1) = M_(1, 0, -1, 1);
  M_(2, 0, 1, -1) = csc(-1.0, M_(0, 2, 1, -1));
  M_(0, 2, -1, 1) = csc(-1.0, M_(2, 0, -1, 1));
  aux = csc(-ctj1, cadd(tjrp, csc(-1.0, tjpr)));
  ADD(0, 1, 1, -1, 1.0, aux); ADD(0, 1, -1, 1, -1.0, aux); ADD(1, 0, 1, -1, -1.0, aux); ADD(1, 0, -1, 1, 1.0, aux);
  ADD(0, 2, 1, -1, 1.0, aux); ADD(0, 2, -1, 1, 1.0, aux); ADD(2, 0, 1, -1, 1.0, aux); ADD(2, 0, -1, 1, 1.0, aux);
  aux = cmk(t0.i, -t0.r);
  ADD(0, 1, 1, -1, 1.0, aux); ADD(0, 1, -1, 1, 1.0, aux); ADD(1, 0, 1, -1, -1.0, aux); ADD(1, 0, -1, 1, -1.0, aux);
  ADD(0, 2, 1, -1, 1.0, aux); ADD(0, 2, -1, 1, -1.0, aux); ADD(2, 0, 1, -1, 1.0, aux); ADD(2, 0, -1, 1, -1.0, aux);
  aux = csc(-0.5 * ctj2, cadd(tjrp, tjpr));
  ADD(0, 1, 1, -1, 1.0, aux); ADD(0, 1, -1, 1, -1.0, aux); ADD(1, 0, 1, -1, -1.0, aux); ADD(1, 0, -1, 1, 1.0, aux);
  ADD(0, 2, 1, -1, -1.0, aux); ADD(0, 2, -1, 1, -1.0, aux); ADD(2, 0, 1, -1, -1.0, aux); ADD(2, 0, -1, 1, -1.0, aux);
  aux = cmk(-ctj2 * (-2.0 * tjrr.i + tjpp.i + tjzz.i) / 3.0, ctj2 * (-2.0 * tjrr.r + tjpp.r + tjzz.r) / 3.0);
  ADD(0, 1, 1, -1, 1.0, aux); ADD(0, 1, -1, 1, 1.0, aux); ADD(1, 0, 1, -1, -1.0, aux); ADD(1, 0, -1, 1, -1.0, aux);
  aux = cmk(-ctj2 * (tjrr.i - 2.0 * tjpp.i + tjzz.i) / 3.0, ctj2 * (tjrr.r - 2.0 * tjpp.r + tjzz.r) / 3.0);
  ADD(0, 2, 1, -1, 1.0, aux); ADD(0, 2, -1, 1, -1.0, aux); ADD(2, 0, 1, -1, 1.0, aux); ADD(2, 0, -1, 1, -1.0, aux);

  M_(0, 3, 1, -1) = csc(csdj, jp);
  M_(0, 3, -1, 1) = M_(0, 3, 1, -1);
  aux = cmk(-csdj * jr.i, csdj * jr.r);
  ADD(0, 3, 1, -1, 1.0, aux); ADD(0, 3, -1, 1, -1.0, aux);
  M_(3, 0, 1, -1) = M_(0, 3, 1, -1);
  M_(3, 0, -1, 1) = M_(0, 3, -1, 1);
  aux = cmk(t1a.i + 0.5 * t2a.i, -t1a.r - 0.5 * t2a.r);
  ADD(0, 3, 1, -1, 1.0, aux); ADD(0, 3, -1, 1, 1.0, aux); ADD(3, 0, 1, -1, -1.0, aux); ADD(3, 0, -1, 1, -1.0, aux);
  aux = cadd(t1b, csc(-0.5, t2b));
  ADD(0, 3, 1, -1, 1.0, aux); ADD(0, 3, -1, 1, -1.0, aux); ADD(3, 0, 1, -1, -1.0, aux); ADD(3, 0, -1, 1, 1.0, aux);

  M_(0, 4, 1, -1) = csc(2.0 * cds, sr);
  M_(0, 4, -1, 1) = M_(0, 4, 1, -1);
  aux = cmk(2.0 * cds * sp.i, -2.0 * cds * sp.r);
  ADD(0, 4, 1, -1, 1.0, aux); ADD(0, 4, -1, 1, -1.0, aux);
  M_(4, 0, 1, -1) = M_(0, 4, 1, -1);
  M_(4, 0, -1, 1) = M_(0, 4, -1, 1);

  M_(1, 2, 1, -1) = cmk(-0.5 * cf * sp.i, 0.5 * cf * sp.r);
  M_(1, 2, -1, 1) = M_(1, 2, 1, -1);
  aux = csc(0.5 * cf, sr);
  ADD(1, 2, 1, -1, 1.0, aux); ADD(1, 2, -1, 1, -1.0, aux);
  M_(2, 1, 1, -1) = csc(-1.0, M_(1, 2, 1, -1));
  M_(2, 1, -1, 1) = csc(-1.0, M_(1, 2, -1, 1));

  M_(1, 3, 1, -1) = csc(0.5 * cf, sz);
  M_(1, 3, -1, 1) = M_(1, 3, 1, -1);
  aux = csc(crdj, rho);
  ADD(1, 3, 1, -1, 1.0, aux); ADD(1, 3, -1, 1, -1.0, aux);
  M_(3, 1, 1, -1) = M_(1, 3, -1, 1);
  M_(3, 1, -1, 1) = M_(1, 3, 1, -1);
  M_(3, 2, 1, -1) = M_(3, 1, 1, -1);
  M_(2, 3, -1, 1) = M_(1, 3, -1, 1);
  M_(2, 3, 1, -1) = csc(-1.0, M_(1, 3, 1, -1));
  M_(3, 2, -1, 1) = csc(-1.0, M_(3, 1, -1, 1));

  M_(3, 3, 1, -1) = csc(ct + 4.0 * cds, sr);
  M_(3, 3, -1, 1) = M_(3, 3, 1, -1);
  aux = cmk((ct + 4.0 * cds) * sp.i, -(ct + 4.0 * cds) * sp.r);
  ADD(3, 3, 1, -1, 1.0, aux); ADD(3, 3, -1, 1, -1.0, aux);
  M_(1, 1, 1, -1) = M_(3, 3, 1, -1);
  M_(1, 1, -1, 1) = M_(3, 3, -1, 1);
  aux = csc(cf, sr);
  ADD(1, 1, 1, -1, 1.0, aux); ADD(1, 1, -1, 1, 1.0, aux);
  M_(2, 2, 1, -1) = M_(3, 3, 1, -1);
  M_(2, 2, -1, 1) = M_(3, 3, -1, 1);
  aux = cmk(cf * sp.i, -cf * sp.r);
  ADD(2, 2, 1, -1, 1.0, aux); ADD(2, 2, -1, 1, -1.0, aux);
#undef ADD
#undef M_
  // pairing fields (pnfam_hamiltonian_blas.f90:1201-1208): index (sa, sb)
  const cplx rb = d[D_RB], sbr = d[D_SBR], sbp = d[D_SBP], sbz = d[D_SBZ];
  mf[100] = cmk(cspair * (sbr.r + sbp.i), cspair * (sbr.i - sbp.r));        // a+ b+
  mf[101] = cmk(cpair * rb.r - cspair * sbz.r, cpair * rb.i - cspair * sbz.i); // a+ b-
  mf[102] = cmk(-cpair * rb.r - cspair * sbz.r, -cpair * rb.i - cspair * sbz.i); // a- b+
  mf[103] = cmk(cspair * (-sbr.r + sbp.i), cspair * (-sbr.i - sbp.r));      // a- b-
  T* out = mfout + ((long long)p * 2 + call) * NMF * 2 * nghl;
  for (int k = 0; k < NMF; ++k) {
    out[((long long)k * 2) * nghl + r] = (T)mf[k].r;
    out[((long long)k * 2 + 1) * nghl + r] = (T)mf[k].i;
  }
}

// ---------------------------------------------------------------------------
// field projection: out_ab = 2 sum_r sum_iy phi_iy(a,r) hpsi(iy)(r,b)
// ---------------------------------------------------------------------------
struct HTask {
  int ix, iy;      // block row / column
  int a0, na;      // row tile inside block ix (spin-uniform)
  int b0, nbc;     // column tile inside block iy
  int sa;          // spin of the rows (+1/-1)
  int mode;        // 0: mean field (5 components), 1: pairing (1 component)
  int call;        // 0: pn, 1: np
  int outq;        // HSP quadrant 0..3 (m11, m12, m21, m22)
  long long ooff;  // block offset inside the quadrant
};

#define HRC 16   // mesh points per K chunk

// grid (ntasks, P); 256 threads (16x16, 2x2 outputs each); dynamic smem
template <class T>
__global__ void __launch_bounds__(256) k_hproj(DevBasisT<T> B, const HTask* __restrict__ tasks,
                                               const T* __restrict__ mf, T* __restrict__ hsp,
                                               long long nxy, const int* __restrict__ active) {
  const int p = blockIdx.y;
  if (!active[p]) return;
  const HTask Th = tasks[blockIdx.x];
  const int nghl = B.nghl;
  const long long ps = (long long)B.dqp * nghl;
  const int nc = Th.mode == 0 ? 5 : 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sA = reinterpret_cast<T*>(smraw);     // [5][32][HRC]
  T* sPb = sA + 5 * 32 * HRC;               // [5][32][HRC]
  T* sMF = sPb + 5 * 32 * HRC;              // [25][2 sb][2 re/im][HRC]
  T* sH = sMF + 25 * 2 * 2 * HRC;           // [5][32][2][HRC]
  __shared__ signed char sns[32];
  const int ja0 = B.st[Th.ix] + Th.a0, jb0 = B.st[Th.iy] + Th.b0;
  if (threadIdx.x < 32) sns[threadIdx.x] = threadIdx.x < Th.nbc ? B.ns[jb0 + threadIdx.x] : (signed char)1;
  const T* mfp = mf + ((long long)p * 2 + Th.call) * NMF * 2 * nghl;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  T ar[2][2] = {{0, 0}, {0, 0}}, ai[2][2] = {{0, 0}, {0, 0}};
  for (int r0 = 0; r0 < nghl; r0 += HRC) {
    const int nr = min(HRC, nghl - r0);
    __syncthreads();
    for (int e = threadIdx.x; e < nc * 32 * HRC; e += 256) {
      const int q = e / (32 * HRC), rem = e % (32 * HRC), aa = rem / HRC, rr = rem % HRC;
      T va = 0, vb = 0;
      if (rr < nr) {
        if (aa < Th.na) va = B.phi[q * ps + (long long)(ja0 + aa) * nghl + r0 + rr];
        if (aa < Th.nbc) vb = B.phi[q * ps + (long long)(jb0 + aa) * nghl + r0 + rr];
      }
      sA[(q * 32 + aa) * HRC + rr] = va;
      sPb[(q * 32 + aa) * HRC + rr] = vb;
    }
    if (Th.mode == 0) {
      for (int e = threadIdx.x; e < 25 * 2 * 2 * HRC; e += 256) {
        const int pair = e / (4 * HRC), rem = e % (4 * HRC), sb = rem / (2 * HRC), rem2 = rem % (2 * HRC);
        const int ri = rem2 / HRC, rr = rem2 % HRC;
        const int iy = pair / 5, iz = pair % 5;
        T v = 0;
        if (rr < nr) v = mfp[((long long)mfslot(iy, iz, Th.sa, sb == 0 ? 1 : -1) * 2 + ri) * nghl + r0 + rr];
        sMF[e] = v;
      }
    } else {
      for (int e = threadIdx.x; e < 2 * 2 * HRC; e += 256) {
        const int sb = e / (2 * HRC), rem = e % (2 * HRC), ri = rem / HRC, rr = rem % HRC;
        const int slot = 100 + (Th.sa < 0 ? 2 : 0) + sb;
        sMF[e] = rr < nr ? mfp[((long long)slot * 2 + ri) * nghl + r0 + rr] : (T)0;
      }
    }
    __syncthreads();
    // hpsi(iy, b, r) = sum_iz mf(iy, iz, sa, s_b)(r) phi_iz(b, r)
    for (int e = threadIdx.x; e < nc * 32 * HRC; e += 256) {
      const int iy = e / (32 * HRC), rem = e % (32 * HRC), bb = rem / HRC, rr = rem % HRC;
      const int sb = sns[bb] > 0 ? 0 : 1;
      T hr = 0, hi = 0;
      if (Th.mode == 0) {
#pragma unroll
        for (int iz = 0; iz < 5; ++iz) {
          const T f = sPb[(iz * 32 + bb) * HRC + rr];
          const T* m = &sMF[((iy * 5 + iz) * 4 + sb * 2) * HRC];
          hr = fma(m[rr], f, hr); hi = fma(m[HRC + rr], f, hi);
        }
      } else {
        const T f = sPb[bb * HRC + rr];
        hr = sMF[(sb * 2) * HRC + rr] * f; hi = sMF[(sb * 2 + 1) * HRC + rr] * f;
      }
      sH[((iy * 32 + bb) * 2) * HRC + rr] = hr;
      sH[((iy * 32 + bb) * 2 + 1) * HRC + rr] = hi;
    }
    __syncthreads();
    for (int q = 0; q < nc; ++q) {
      for (int rr = 0; rr < HRC; ++rr) {
        const T a0 = sA[(q * 32 + ty * 2) * HRC + rr], a1 = sA[(q * 32 + ty * 2 + 1) * HRC + rr];
        const T h0r = sH[((q * 32 + tx * 2) * 2) * HRC + rr], h0i = sH[((q * 32 + tx * 2) * 2 + 1) * HRC + rr];
        const T h1r = sH[((q * 32 + tx * 2 + 1) * 2) * HRC + rr], h1i = sH[((q * 32 + tx * 2 + 1) * 2 + 1) * HRC + rr];
        ar[0][0] = fma(a0, h0r, ar[0][0]); ai[0][0] = fma(a0, h0i, ai[0][0]);
        ar[0][1] = fma(a0, h1r, ar[0][1]); ai[0][1] = fma(a0, h1i, ai[0][1]);
        ar[1][0] = fma(a1, h0r, ar[1][0]); ai[1][0] = fma(a1, h0i, ai[1][0]);
        ar[1][1] = fma(a1, h1r, ar[1][1]); ai[1][1] = fma(a1, h1i, ai[1][1]);
      }
    }
  }
  const int ld = B.db[Th.ix];
  T* ore = hsp + ((long long)p * 2 + 0) * 4 * nxy + (long long)Th.outq * nxy + Th.ooff;
  T* oim = hsp + ((long long)p * 2 + 1) * 4 * nxy + (long long)Th.outq * nxy + Th.ooff;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int a = ty * 2 + i, b = tx * 2 + j;
      if (a < Th.na && b < Th.nbc) {
        const long long e = (Th.a0 + a) + (long long)(Th.b0 + b) * ld;
        ore[e] = (T)2 * ar[i][j];
        oim[e] = (T)2 * ai[i][j];
      }
    }
}

// ---------------------------------------------------------------------------
// Green's function update: vout = G o (q*H + F); layout [P][Re X|Y, Im X|Y]
// ---------------------------------------------------------------------------
// corr[p] != 0 (increment step of the mixed form, H evaluated from X - X_anchor):
// vout = G o (q*H) + radd[p], radd = g(X_anchor) evaluated in FP64
__global__ void k_green(long long nxy, int P, const double* __restrict__ hqp, const double* __restrict__ fqp,
                        const int* __restrict__ erow, const int* __restrict__ ecol,
                        const double* __restrict__ E1, const double* __restrict__ E2,
                        const double* __restrict__ wre, const double* __restrict__ wim, double quench,
                        double* __restrict__ vout, const int* __restrict__ active,
                        const int* __restrict__ corr, const double* __restrict__ radd) {
  const int p = blockIdx.y;
  if (!active[p]) return;
  const long long n2 = 2 * nxy;
  const double wr = wre[p], wi = wim[p];
  const bool cstep = corr && corr[p];
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n2; e += (long long)gridDim.x * blockDim.x) {
    double hr = 0.0, hi = 0.0;
    if (hqp) { hr = quench * hqp[(long long)p * 2 * n2 + e]; hi = quench * hqp[(long long)p * 2 * n2 + n2 + e]; }
    if (!cstep) hr += fqp[e];
    // G = -1/(E1 + E2 -/+ w): X (e < nxy) uses -w, Y uses +w
    const double sgn = e < nxy ? -1.0 : 1.0;
    const double dr = E1[erow[e]] + E2[ecol[e]] + sgn * wr, di = sgn * wi;
    const double den = dr * dr + di * di;
    const double gr = -dr / den, gi = di / den;
    double vr = gr * hr - gi * hi, vi = gr * hi + gi * hr;
    if (cstep) { vr += radd[(long long)p * 2 * n2 + e]; vi += radd[(long long)p * 2 * n2 + n2 + e]; }
    vout[(long long)p * 2 * n2 + e] = vr;
    vout[(long long)p * 2 * n2 + n2 + e] = vi;
  }
}

// ---------------------------------------------------------------------------
// Broyden mixing on device (pnfam_broyden.f90:117-216), one independent
// history per point: itp[p] is the point's own Broyden iteration number and
// modep[p] what the step does (BRO_* below)
// ---------------------------------------------------------------------------
enum { BRO_BROYDEN = 0, BRO_LINEAR = 1, BRO_NOMIX = 2 };
struct BroState {
  int N;            // vector length (4*nxy)
  int M;            // history size
  double alpha;
  double* vin;      // [P][N]
  double* vout;     // [P][N]
  double* df;       // [P][M][N]
  double* dv;       // [P][M][N]
  double* part;     // [P][nchunk][NPART] block partials
  int nchunk;
  const int* itp;   // [P] Broyden iteration of each point
  const int* modep; // [P] BRO_*
};
enum { BRO_NPART = 2 + 2 * 64 };  // 0: max|vout|, 1: |df_ipos|^2, 2..: dots

// history slots of Broyden iteration `it` (Fortran integer division truncates
// toward zero, as C++ does): iter_used columns in use, ipos the column updated
// this step, inext the column written at the end (0-based)
__host__ __device__ __forceinline__ void bro_slots(int it, int M, int& iter_used, int& ipos, int& inext) {
  iter_used = it - 1 < M ? it - 1 : M;
  ipos = it - 1 - ((it - 2) / M) * M - 1;
  inext = it - ((it - 1) / M) * M - 1;
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  return s;  // valid in thread 0
}
__device__ __forceinline__ double block_max(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s = fmax(s, sh[i]);
  return s;
}

// vout -= vin; max|vout|; history column ipos: df = vout - df, dv = vin - dv, |df|^2
__global__ void __launch_bounds__(256) k_bro_diff(BroState S, const int* __restrict__ active) {
  const int p = blockIdx.y;
  if (!active[p]) return;
  __shared__ double sh[32];
  const int it = S.itp[p], mode = S.modep[p];
  int iu, ipos, inext;
  bro_slots(it, S.M, iu, ipos, inext);
  const bool upd = mode == BRO_BROYDEN && it >= 2;
  double* vo = S.vout + (long long)p * S.N;
  const double* vi = S.vin + (long long)p * S.N;
  double* df = upd ? S.df + ((long long)p * S.M + ipos) * S.N : nullptr;
  double* dv = upd ? S.dv + ((long long)p * S.M + ipos) * S.N : nullptr;
  double mx = 0.0, nn = 0.0;
  const int chunk = (S.N + S.nchunk - 1) / S.nchunk;
  const int e0 = blockIdx.x * chunk, e1 = min(S.N, e0 + chunk);
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const double v = vo[e] - vi[e];
    vo[e] = v;
    mx = fmax(mx, fabs(v));
    if (upd) {
      const double f = v - df[e];
      df[e] = f;
      dv[e] = vi[e] - dv[e];
      nn = fma(f, f, nn);
    }
  }
  const double m = block_max(mx, sh);
  const double s = block_sum(nn, sh);
  if (threadIdx.x == 0) {
    double* pt = S.part + ((long long)p * S.nchunk + blockIdx.x) * BRO_NPART;
    pt[0] = m; pt[1] = s;
  }
}

// normalise column ipos by 1/|df_ipos| and form the dots
// dd[k] = df_k . df_ipos and wk[k] = df_k . vout for k < iter_used
__global__ void __launch_bounds__(256) k_bro_dots(BroState S, const double* __restrict__ norm,
                                                  const int* __restrict__ active) {
  const int p = blockIdx.y;
  if (!active[p]) return;
  const int it = S.itp[p], mode = S.modep[p];
  if (mode != BRO_BROYDEN || it < 1) return;
  int iu, ipos, inext;
  bro_slots(it, S.M, iu, ipos, inext);
  const bool upd = it >= 2;
  __shared__ double sh[32];
  const double* vo = S.vout + (long long)p * S.N;
  const int chunk = (S.N + S.nchunk - 1) / S.nchunk;
  const int e0 = blockIdx.x * chunk, e1 = min(S.N, e0 + chunk);
  double* dfp = S.df + (long long)p * S.M * S.N;
  double* dvp = S.dv + (long long)p * S.M * S.N;
  if (upd) {
    const double sc = norm[p];
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      dfp[(long long)ipos * S.N + e] *= sc;
      dvp[(long long)ipos * S.N + e] *= sc;
    }
  }
  __syncthreads();
  double* pt = S.part + ((long long)p * S.nchunk + blockIdx.x) * BRO_NPART;
  for (int k = 0; k < iu; ++k) {
    double a = 0.0, b = 0.0;
    const double* fk = dfp + (long long)k * S.N;
    const double* fi = dfp + (long long)ipos * S.N;
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      a = fma(fk[e], fi[e], a);
      b = fma(fk[e], vo[e], b);
    }
    const double sa = block_sum(a, sh);
    const double sb = block_sum(b, sh);
    if (threadIdx.x == 0) { pt[2 + k] = sa; pt[2 + 64 + k] = sb; }
  }
}

// one CTA per point: reduce partials; stage 0: si and 1/|df_ipos|; stage 1:
// maintain beta (M x M) and solve beta*gamma = work
__global__ void k_bro_solve(BroState S, int stage, double w0, double* __restrict__ si, double* __restrict__ norm,
                            double* __restrict__ beta, double* __restrict__ gamma, const int* __restrict__ active) {
  const int p = blockIdx.x;
  if (!active[p]) return;
  const double* pt = S.part + (long long)p * S.nchunk * BRO_NPART;
  if (stage == 0) {
    if (threadIdx.x == 0) {
      double m = 0.0, s = 0.0;
      for (int c = 0; c < S.nchunk; ++c) { m = fmax(m, pt[c * BRO_NPART]); s += pt[c * BRO_NPART + 1]; }
      si[p] = m;
      norm[p] = s > 0.0 ? 1.0 / sqrt(s) : 0.0;
    }
    return;
  }
  const int it = S.itp[p], mode = S.modep[p];
  if (mode != BRO_BROYDEN || it < 1) return;
  int n, ipos, inext;
  bro_slots(it, S.M, n, ipos, inext);
  __shared__ double A[64][65];
  __shared__ double x[64];
  const int M = S.M;
  double* bp = beta + (long long)p * M * M;
  if (threadIdx.x == 0) {
    for (int k = 0; k < n; ++k) {
      double dd = 0.0, wk = 0.0;
      for (int c = 0; c < S.nchunk; ++c) { dd += pt[c * BRO_NPART + 2 + k]; wk += pt[c * BRO_NPART + 2 + 64 + k]; }
      if (k != ipos) { bp[k * M + ipos] = dd; bp[ipos * M + k] = dd; }
      x[k] = wk;
    }
    for (int k = 0; k < n; ++k) bp[k * M + k] = w0 * w0 + 1.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) A[i][j] = bp[i * M + j];
    // Gaussian elimination with partial pivoting
    for (int c = 0; c < n; ++c) {
      int piv = c;
      for (int r = c + 1; r < n; ++r) if (fabs(A[r][c]) > fabs(A[piv][c])) piv = r;
      if (piv != c) {
        for (int j = 0; j < n; ++j) { const double t = A[c][j]; A[c][j] = A[piv][j]; A[piv][j] = t; }
        const double t = x[c]; x[c] = x[piv]; x[piv] = t;
      }
      for (int r = c + 1; r < n; ++r) {
        const double f = A[r][c] / A[c][c];
        for (int j = c; j < n; ++j) A[r][j] -= f * A[c][j];
        x[r] -= f * x[c];
      }
    }
    for (int r = n - 1; r >= 0; --r) {
      double s = x[r];
      for (int j = r + 1; j < n; ++j) s -= A[r][j] * x[j];
      x[r] = s / A[r][r];
    }
    for (int k = 0; k < n; ++k) gamma[(long long)p * 64 + k] = x[k];
  }
}

// BRO_BROYDEN: curv = alpha*vout - sum_i gamma_i (dv_i + alpha df_i);
//              df[inext] = vout; dv[inext] = vin; vin += curv
// BRO_LINEAR:  vin += alpha*vout;  BRO_NOMIX: vin += vout
__global__ void __launch_bounds__(256) k_bro_update(BroState S, const double* __restrict__ gamma,
                                                    const int* __restrict__ active) {
  const int p = blockIdx.y;
  if (!active[p]) return;
  const int it = S.itp[p], mode = S.modep[p];
  int iu, ipos, inext;
  bro_slots(it, S.M, iu, ipos, inext);
  if (mode != BRO_BROYDEN) iu = 0;
  double* vi = S.vin + (long long)p * S.N;
  const double* vo = S.vout + (long long)p * S.N;
  __shared__ double g[64];
  if (mode == BRO_BROYDEN && (int)threadIdx.x < iu) g[threadIdx.x] = gamma[(long long)p * 64 + threadIdx.x];
  __syncthreads();
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < S.N; e += (long long)gridDim.x * blockDim.x) {
    const double v = vo[e];
    if (mode == BRO_NOMIX) { vi[e] += v; continue; }
    if (mode == BRO_LINEAR) { vi[e] += S.alpha * v; continue; }
    double c = S.alpha * v;
    const double* dfp = S.df + (long long)p * S.M * S.N;
    const double* dvp = S.dv + (long long)p * S.M * S.N;
    for (int k = 0; k < iu; ++k)
      c -= g[k] * (dvp[(long long)k * S.N + e] + S.alpha * dfp[(long long)k * S.N + e]);
    const double old = vi[e];
    S.df[((long long)p * S.M + inext) * S.N + e] = v;
    S.dv[((long long)p * S.M + inext) * S.N + e] = old;
    vi[e] = old + c;
  }
}

// per-point vector operations, [P][n] layout:
// op 0: dst = src; op 1: dst += src; op 2: dst = 0; op 3: dst = a*src
__global__ void k_vecop(int op, double a, double* __restrict__ dst, const double* __restrict__ src, long long n,
                        const int* __restrict__ mask) {
  const int p = blockIdx.y;
  if (!mask[p]) return;
  double* d = dst + (long long)p * n;
  const double* s_ = src ? src + (long long)p * n : nullptr;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    if (op == 0) d[e] = s_[e];
    else if (op == 1) d[e] += s_[e];
    else if (op == 2) d[e] = 0.0;
    else d[e] = a * s_[e];
  }
}

// S_k = -1/pi * (F_k . Re, F_k . Im) for the operator (k=0) and cross terms
// fops: [nops][2*nxy]; part: [P][nchunk][2*nops]
__global__ void __launch_bounds__(256) k_contract(long long nxy, int nops, const double* __restrict__ fops,
                                                  const double* __restrict__ vin, int nchunk,
                                                  double* __restrict__ part, const int* __restrict__ active) {
  const int p = blockIdx.y;
  if (!active[p]) return;
  __shared__ double sh[32];
  const long long n2 = 2 * nxy;
  const double* v = vin + (long long)p * 2 * n2;
  const long long chunk = (n2 + nchunk - 1) / nchunk;
  const long long e0 = blockIdx.x * chunk, e1 = min(n2, e0 + chunk);
  for (int k = 0; k < nops; ++k) {
    double a = 0.0, b = 0.0;
    for (long long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      const double f = fops[(long long)k * n2 + e];
      a = fma(f, v[e], a);
      b = fma(f, v[n2 + e], b);
    }
    const double sa = block_sum(a, sh);
    const double sb = block_sum(b, sh);
    if (threadIdx.x == 0) {
      part[((long long)p * nchunk + blockIdx.x) * 2 * nops + 2 * k] = sa;
      part[((long long)p * nchunk + blockIdx.x) * 2 * nops + 2 * k + 1] = sb;
    }
  }
}

}  // namespace pnfam

namespace pnfam {
// per-point precision conversions: out[p*n + e] = in[p*n + e] for points with act[p]
// (act == nullptr: all points)
// out = (float)(in - sub), sub optional; with dmax, dmax[p] = max(dmax[p], max|in - sub|)
// (dmax as the bit pattern of a non-negative double, which orders like the integer)
__global__ void __launch_bounds__(256) k_to_f32(const double* __restrict__ in, float* __restrict__ out, long long n,
                                                int P, long long ld, const int* __restrict__ act,
                                                const double* __restrict__ sub = nullptr,
                                                unsigned long long* __restrict__ dmax = nullptr) {
  const int p = blockIdx.y;
  if (act && !act[p]) return;
  double m = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const double v = sub ? in[p * ld + e] - sub[p * ld + e] : in[p * ld + e];
    m = fmax(m, fabs(v));
    out[p * ld + e] = (float)v;
  }
  if (dmax) {
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(dmax + p, (unsigned long long)__double_as_longlong(m));
  }
}
__global__ void k_to_f64(const float* __restrict__ in, double* __restrict__ out, long long n, long long ld,
                         const int* __restrict__ act) {
  const int p = blockIdx.y;
  if (act && !act[p]) return;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    out[p * ld + e] = (double)in[p * ld + e];
}
}  // namespace pnfam
