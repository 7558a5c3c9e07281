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

#include "tc.cuh"

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
  int tm, pad_;        // tile shape: tm rows x 1024 / tm columns (tm = 8 ... 128)
};

#define GT 32
#define GK 16

template <class T>
__device__ __forceinline__ const T* bufptr(const BufDescT<T>* b, int id, int p, int plane, long long off) {
  const BufDescT<T> d = b[id];
  return d.base + (long long)p * d.sp + (long long)plane * d.spl + off;
}

// C = sum_t alpha_t op(A_t) op(B_t); blockIdx.y = point*2 + plane; T = compute type.
// Output tiles of TM x TN = 1024 elements (TM = 8 ... 128, chosen per task from its M
// and N), 2 x 2 per thread; every element sums over k in the same order whatever the
// shape.
template <class T, int TM>
__device__ __forceinline__ void gemm_tile(const GemmTask& Tk, int lt, const BufDescT<T>* __restrict__ bufs, int p,
                                          int plane, T* smem) {
  constexpr int TN = 1024 / TM, TX = TN / 2;
  T* As = smem;                    // [GK][TM + 1]
  T* Bs = smem + GK * (TM + 1);    // [GK][TN + 1]
  const int m0 = (lt / Tk.ntn) * TM, n0 = (lt % Tk.ntn) * TN;
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  T acc00 = 0, acc01 = 0, acc10 = 0, acc11 = 0;
  const int M = Tk.M, N = Tk.N, K = Tk.K;
  for (int it = 0; it < Tk.nterm; ++it) {
    const GemmTerm& tm = Tk.t[it];
    const T* A = bufptr(bufs, tm.abuf, p, plane, tm.aoff);
    const T* B = bufptr(bufs, tm.bbuf, p, plane, tm.boff);
    const T alpha = (T)tm.alpha[plane];
    for (int k0 = 0; k0 < K; k0 += GK) {
      for (int e = threadIdx.x; e < GK * TM; e += 256) {
        const int kk = e / TM, mm = e % TM;
        const int gm = m0 + mm, gk = k0 + kk;
        T v = 0;
        if (gm < M && gk < K) v = tm.tA ? A[gk + (long long)gm * tm.lda] : A[gm + (long long)gk * tm.lda];
        As[kk * (TM + 1) + mm] = alpha * v;
      }
      for (int e = threadIdx.x; e < GK * TN; e += 256) {
        const int kk = e / TN, nn = e % TN;
        const int gn = n0 + nn, gk = k0 + kk;
        T w = 0;
        if (gn < N && gk < K) w = tm.tB ? B[gn + (long long)gk * tm.ldb] : B[gk + (long long)gn * tm.ldb];
        Bs[kk * (TN + 1) + nn] = w;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < GK; ++kk) {
        const T a0 = As[kk * (TM + 1) + ty * 2], a1 = As[kk * (TM + 1) + ty * 2 + 1];
        const T b0 = Bs[kk * (TN + 1) + tx * 2], b1 = Bs[kk * (TN + 1) + tx * 2 + 1];
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

template <class T>
__global__ void __launch_bounds__(256) k_gemm(const GemmTask* __restrict__ tasks, const int* __restrict__ tile2task,
                                              const BufDescT<T>* __restrict__ bufs, const int* __restrict__ active) {
  const int z = blockIdx.y;
  const int p = z >> 1, plane = z & 1;
  if (active && !active[p]) return;
  const int tile = blockIdx.x;
  const GemmTask& Tk = tasks[tile2task[tile]];
  const int lt = tile - Tk.tile0;
  __shared__ T smem[GK * (128 + 1) + GK * (8 + 1)];
  switch (Tk.tm) {
    case 8: gemm_tile<T, 8>(Tk, lt, bufs, p, plane, smem); break;
    case 16: gemm_tile<T, 16>(Tk, lt, bufs, p, plane, smem); break;
    case 64: gemm_tile<T, 64>(Tk, lt, bufs, p, plane, smem); break;
    case 128: gemm_tile<T, 128>(Tk, lt, bufs, p, plane, smem); break;
    default: gemm_tile<T, 32>(Tk, lt, bufs, p, plane, smem); break;
  }
}

// ---------------------------------------------------------------------------
// grouped block GEMM on the tensor cores (FP32 data, 3xTF32 products).
// Every term multiplies a per-point block (state, intermediate, field) by a
// ground-state block (U or V) shared by all points.  The per-point operand is
// put on the M side of the MMA so that the rows of all active points and both
// planes (Re, Im) fill 128-row tiles:
//   case 0 (per-point operand on the left):  D[i][j] = C[i][j],  D = op(P) op(S)
//   case 1 (per-point operand on the right): D[j][i] = C[i][j],  D = op(P)^T op(S)^T
// Rows: (point, plane, i) with i fastest; columns padded to a multiple of 16.
// ---------------------------------------------------------------------------
struct GemmTaskTC {
  int M, N, K, nterm;
  int rcase;              // 0 or 1, as above
  int mrows, ncols, npad; // D rows per (point, plane), D columns, padded columns
  GemmTerm t[PNFAM_MAXTERM];
  long long coff;
  int cbuf, ldc;
  long long bsoff;        // floats: the task's ground-state operand, split and laid out per chunk
};
enum { GTC_K = 16, GTC_PROD = 256, GTC_THREADS = GTC_PROD + 32 };

// two stages sized for the widest padded block (npmax <= 256) of the launch's tasks:
// narrower task lists leave room for more CTAs per SM, so more loads are in flight
__host__ __device__ constexpr size_t gemm_tc_smem_bytes(int npmax = 256) {
  return (size_t)2 * (2 * 128 * GTC_K + 2 * npmax * GTC_K) * sizeof(float);
}

// the B tile of chunk c of a task: B[n][k] = op(S)[k0 + k][n] (case 0) or
// op(S)[n][k0 + k] (case 1), n < ncols, zero elsewhere
__device__ __forceinline__ float4 gemm_tc_b4(const GemmTaskTC& Tk, const BufDescT<float>* bufs, int c, int n, int k4) {
  const int nkc = (Tk.K + GTC_K - 1) / GTC_K;
  const GemmTerm& tm = Tk.t[c / nkc];
  const int k0 = (c % nkc) * GTC_K;
  const bool pa = Tk.rcase == 0;
  const int sbuf = pa ? tm.bbuf : tm.abuf;
  const long long soff = pa ? tm.boff : tm.aoff;
  const int sld = pa ? tm.ldb : tm.lda, str_ = pa ? tm.tB : tm.tA;
  float x[4] = {0.f, 0.f, 0.f, 0.f};
  if (n < Tk.ncols) {
    const float* S = bufs[sbuf].base + soff;
    const bool kfast = pa ? str_ == 0 : str_ != 0;
    const long long sn = kfast ? sld : 1, sk = kfast ? 1 : sld;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int k = k0 + 4 * k4 + u;
      if (k < Tk.K) x[u] = S[(long long)n * sn + (long long)k * sk];
    }
  }
  return make_float4(x[0], x[1], x[2], x[3]);
}

// the ground-state operand of every chunk of every task, split into TF32 hi and lo
// in the canonical layout, once per operator: gsplit[bsoff + c*npad*2*GTC_K] = hi | lo
// grid (ntasks, most chunks of a task), 256 threads
__global__ void __launch_bounds__(256) k_gemm_bsplit(const GemmTaskTC* __restrict__ tasks,
                                                     const BufDescT<float>* __restrict__ bufs,
                                                     float* __restrict__ gsplit) {
  const GemmTaskTC& Tk = tasks[blockIdx.x];
  const int c = blockIdx.y;
  if (c >= Tk.nterm * ((Tk.K + GTC_K - 1) / GTC_K)) return;
  const int NP = Tk.npad;
  float* dst = gsplit + Tk.bsoff + (long long)c * NP * 2 * GTC_K;
  for (int e = threadIdx.x; e < NP * (GTC_K / 4); e += blockDim.x) {
    const int n = e % NP, k4 = e / NP;
    const int o = tc::cm_off(n, 4 * k4, NP);
    st_split4(dst + o, dst + NP * GTC_K + o, gemm_tc_b4(Tk, bufs, c, n, k4));
  }
}

// grid (ntasks, row tiles of 128); GTC_THREADS threads; dynamic smem gemm_tc_smem_bytes(npmax),
// npmax >= every task's npad
__global__ void __launch_bounds__(GTC_THREADS, 2) k_gemm_tc(const GemmTaskTC* __restrict__ tasks,
                                                            const BufDescT<float>* __restrict__ bufs,
                                                            const float* __restrict__ gsplit,
                                                            const int* __restrict__ actlist, int nact,
                                                            int npmax, int* __restrict__ err) {
  const GemmTaskTC& Tk = tasks[blockIdx.x];
  const int rows_total = 2 * nact * Tk.mrows;
  const int R0 = blockIdx.y * 128;
  if (R0 >= rows_total) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  float* stage_base = reinterpret_cast<float*>(smraw);
  const int stage_floats = 2 * 128 * GTC_K + 2 * npmax * GTC_K;
  __shared__ __align__(8) uint64_t full_bar[2], empty_bar[2];
  __shared__ uint32_t tslot;
  __shared__ volatile int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int NP = Tk.npad, K = Tk.K, mr = Tk.mrows;
  const int nkc = (K + GTC_K - 1) / GTC_K;
  const int nchunk = Tk.nterm * nkc;
  const uint32_t ncols = NP <= 32 ? 32u : NP <= 64 ? 64u : NP <= 128 ? 128u : 256u;
  if (tid == 0) {
    tc::mbar_init(&full_bar[0], GTC_PROD); tc::mbar_init(&full_bar[1], GTC_PROD);
    tc::mbar_init(&empty_bar[0], 1); tc::mbar_init(&empty_bar[1], 1);
    abort_flag = 0;
  }
  if (warp == 0) tc::tmem_alloc(&tslot, ncols);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tslot;
  if (warp < GTC_PROD / 32) {
    // ---------------- producers ----------------
    int lc0 = -1, lc1 = -1;   // thread 0: last chunk copied into stage 0, stage 1
    for (int c = 0; c < nchunk; ++c) {
      const int st = c & 1;
      if (c >= 2 && !abort_flag && !tc::mbar_wait(&empty_bar[st], ((c >> 1) - 1) & 1)) abort_flag = 1;
      float* sAh = stage_base + st * stage_floats;
      float* sAl = sAh + 128 * GTC_K;
      float* sBh = sAl + 128 * GTC_K;
      bool issued = false;
      if (tid == 0 && !abort_flag) {
        // B: the ground-state operand of this chunk, pre-split (hi then lo, NP x GTC_K
        // each); this thread's arrival on the stage comes with the copy
        const uint32_t bbytes = (uint32_t)NP * GTC_K * 2 * 4;
        tc::mbar_expect_tx(&full_bar[st], bbytes);
        tc::bulk_g2s(sBh, gsplit + Tk.bsoff + (long long)c * NP * 2 * GTC_K, bbytes, &full_bar[st]);
        issued = true;
        if (st == 0) lc0 = c; else lc1 = c;
      }
      const GemmTerm& tm = Tk.t[c / nkc];
      const int k0 = (c % nkc) * GTC_K;
      // which operand of the term is the per-point one
      const bool pa = Tk.rcase == 0;
      const int pbuf = pa ? tm.abuf : tm.bbuf;
      const long long poff = pa ? tm.aoff : tm.boff;
      const int pld = pa ? tm.lda : tm.ldb;
      const int ptr_ = pa ? tm.tA : tm.tB;
      if (!abort_flag) {
        // A[m][k]: row m = (point, plane, i); case 0: op(P)[i][k], case 1: op(P)[k][i]
        for (int e = tid; e < 128 * (GTC_K / 4); e += GTC_PROD) {
          const int m = e & 127, k4 = e >> 7, R = R0 + m;
          float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
          if (R < rows_total) {
            const int i = R % mr, rest = R / mr, pl = rest & 1, p = actlist[rest >> 1];
            const BufDescT<float> d = bufs[pbuf];
            const float* P = d.base + (long long)p * d.sp + (long long)pl * d.spl + poff;
            const float al = (float)tm.alpha[pl];
            // element (i, k) of op(P) (case 0) or (k, i) of op(P) (case 1): stride in k
            const bool kfast = pa ? ptr_ != 0 : ptr_ == 0;
            const long long si = kfast ? pld : 1, sk = kfast ? 1 : pld;
            float x[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const int k = k0 + 4 * k4 + u;
              x[u] = k < K ? al * P[(long long)i * si + (long long)k * sk] : 0.f;
            }
            v = make_float4(x[0], x[1], x[2], x[3]);
          }
          const int o = tc::cm_off(m, 4 * k4, 128);
          st_split4(sAh + o, sAl + o, v);
        }
      }
      tc::fence_async_smem();
      if (!issued) tc::mbar_arrive(&full_bar[st]);
    }
    // no copy may still be landing when the memory is reused (the last two chunks
    // are the only ones that can be in flight)
    if (tid == 0) {
      if (lc0 >= 0 && !tc::mbar_wait(&full_bar[0], (lc0 >> 1) & 1)) abort_flag = 1;
      if (lc1 >= 0 && !tc::mbar_wait(&full_bar[1], (lc1 >> 1) & 1)) abort_flag = 1;
    }
  } else if (tid == GTC_PROD) {
    // ---------------- MMA issuer ----------------
    const uint32_t idesc = tc::idesc_tf32(128, NP);
    const uint32_t lboA = (128 / 8) * 128, lboB = (uint32_t)(NP / 8) * 128;
    for (int c = 0; c < nchunk; ++c) {
      const int st = c & 1;
      if (!abort_flag && !tc::mbar_wait(&full_bar[st], (c >> 1) & 1)) abort_flag = 1;
      tc::fence_after();
      if (!abort_flag) {
        const float* sAh = stage_base + st * stage_floats;
        const float* sAl = sAh + 128 * GTC_K;
        const float* sBh = sAl + 128 * GTC_K;
        const float* sBl = sBh + NP * GTC_K;
#pragma unroll
        for (int ks = 0; ks < GTC_K / 8; ++ks) {
          const uint32_t oa = ks * 2 * lboA, ob = ks * 2 * lboB;
          const uint64_t ah = tc::sdesc(tc::smem_u32(sAh) + oa, lboA, 128);
          const uint64_t al = tc::sdesc(tc::smem_u32(sAl) + oa, lboA, 128);
          const uint64_t bh = tc::sdesc(tc::smem_u32(sBh) + ob, lboB, 128);
          const uint64_t bl = tc::sdesc(tc::smem_u32(sBl) + ob, lboB, 128);
          tc::mma_tf32(tmem, ah, bh, idesc, c > 0 || ks > 0);
          tc::mma_tf32(tmem, ah, bl, idesc, true);
          tc::mma_tf32(tmem, al, bh, idesc, true);
        }
      }
      tc::mma_commit(&empty_bar[st]);
    }
  }
  const int last = nchunk - 1;
  bool ok = nchunk == 0 || tc::mbar_wait(&empty_bar[last & 1], (last >> 1) & 1);
  ok = __syncthreads_and(ok && !abort_flag);
  tc::fence_after();
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
  } else if (warp < 4) {
    const int m = tid, R = R0 + m;
    const bool mine = R < rows_total;
    const int i = mine ? R % mr : 0, rest = mine ? R / mr : 0, pl = rest & 1;
    const int p = mine ? actlist[rest >> 1] : 0;
    const BufDescT<float> d = bufs[Tk.cbuf];
    float* C = d.base + (long long)p * d.sp + (long long)pl * d.spl + Tk.coff;
    for (int n0 = 0; n0 < NP; n0 += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)n0, v);
      if (mine) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int n = n0 + u;
          if (n < Tk.ncols) {
            if (Tk.rcase == 0) C[i + (long long)n * Tk.ldc] = v[u];
            else C[n + (long long)i * Tk.ldc] = v[u];
          }
        }
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tmem, ncols);
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

// four consecutive elements from shared memory (16-byte aligned) as 128-bit loads
__device__ __forceinline__ void lds4(const float* p, float (&v)[4]) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void lds4(const double* p, double (&v)[4]) {
  const double2 t0 = reinterpret_cast<const double2*>(p)[0], t1 = reinterpret_cast<const double2*>(p)[1];
  v[0] = t0.x; v[1] = t0.y; v[2] = t1.x; v[3] = t1.y;
}

#define DRT 32   // mesh points per CTA

// b columns per thread: 4 consecutive columns per lane, 8 lanes
template <class T> struct DensTile {
  static constexpr int BT = 4;
  static constexpr int BW = 8 * BT;              // b columns per chunk (8 lanes x BT)
  static constexpr int BWP = BW + 4;             // padded row: conflict-free transposed staging
  static constexpr int AK = sizeof(T) >= 8 ? 16 : 32;  // a rows per chunk
};

template <class T>
__host__ __device__ constexpr size_t density_smem_bytes() {
  return (size_t)(DensTile<T>::AK * DRT * 4 + 2 * DensTile<T>::AK * DensTile<T>::BWP) * sizeof(T);
}

// contributions of one column b at one mesh point from the rows of the SAME spin
// as b (S) or of the OPPOSITE spin (O); P = phi_q(b, r), sg = spin of b,
// sig = +1 if b is spin down (pnfam_hamiltonian_blas.f90:124-711)
template <class T>
__device__ __forceinline__ void dens_same(T (&acc)[2 * ND], const T (&Sr)[4], const T (&Si)[4], const T (&P)[4],
                                          T sg) {
  const T h5 = T(0.5);
#define ACC(k, re, im) { acc[2 * (k)] += (re); acc[2 * (k) + 1] += (im); }
  T xr, xi;
  xr = Sr[0] * P[0]; xi = Si[0] * P[0];
  ACC(D_RHO, xr, xi);
  ACC(D_SZ, sg * xr, sg * xi);
  xr = h5 * (Sr[0] * P[2] + Sr[2] * P[0]); xi = h5 * (Si[0] * P[2] + Si[2] * P[0]);
  ACC(D_JP, xr, xi);
  ACC(D_TJPZ, sg * xr, sg * xi);
  xr = Sr[1] * P[1] + Sr[2] * P[2] + Sr[3] * P[3]; xi = Si[1] * P[1] + Si[2] * P[2] + Si[3] * P[3];
  ACC(D_TAU, xr, xi);
  ACC(D_TZ, sg * xr, sg * xi);
  xr = h5 * (Sr[0] * P[1] - Sr[1] * P[0]); xi = h5 * (Si[0] * P[1] - Si[1] * P[0]);
  ACC(D_JR, -xi, xr);
  ACC(D_TJRZ, -sg * xi, sg * xr);
  xr = h5 * (Sr[0] * P[3] - Sr[3] * P[0]); xi = h5 * (Si[0] * P[3] - Si[3] * P[0]);
  ACC(D_JZ, -xi, xr);
  ACC(D_TJZZ, -sg * xi, sg * xr);
  ACC(D_GS, sg * (Sr[0] * P[3] + Sr[3] * P[0]), sg * (Si[0] * P[3] + Si[3] * P[0]));
  ACC(D_FR, h5 * sg * (Sr[1] * P[3] + Sr[3] * P[1]), h5 * sg * (Si[1] * P[3] + Si[3] * P[1]));
  {
    const T ar = h5 * sg * (Sr[2] * P[3] - Sr[3] * P[2]), ai = h5 * sg * (Si[2] * P[3] - Si[3] * P[2]);
    ACC(D_FP, -ai, ar);
  }
  ACC(D_FZ, sg * Sr[3] * P[3], sg * Si[3] * P[3]);
}

template <class T>
__device__ __forceinline__ void dens_opp(T (&acc)[2 * ND], const T (&Or)[4], const T (&Oi)[4], const T (&P)[4],
                                         T sig) {
  const T h5 = T(0.5);
  T xr, xi;
  ACC(D_GS, sig * (Or[0] * P[2] - Or[2] * P[0]) + (Or[0] * P[1] + Or[1] * P[0]),
      sig * (Oi[0] * P[2] - Oi[2] * P[0]) + (Oi[0] * P[1] + Oi[1] * P[0]));
  ACC(D_FR, Or[1] * P[1] + sig * h5 * (Or[1] * P[2] - Or[2] * P[1]),
      Oi[1] * P[1] + sig * h5 * (Oi[1] * P[2] - Oi[2] * P[1]));
  {
    const T ar = sig * Or[2] * P[2] + h5 * (Or[2] * P[1] - Or[1] * P[2]);
    const T ai = sig * Oi[2] * P[2] + h5 * (Oi[2] * P[1] - Oi[1] * P[2]);
    ACC(D_FP, -ai, ar);
  }
  ACC(D_FZ, h5 * (Or[3] * P[1] + sig * Or[3] * P[2] + Or[1] * P[3] - sig * Or[2] * P[3]),
      h5 * (Oi[3] * P[1] + sig * Oi[3] * P[2] + Oi[1] * P[3] - sig * Oi[2] * P[3]));
  xr = Or[0] * P[0]; xi = Oi[0] * P[0];
  ACC(D_SR, xr, xi);
  ACC(D_SP, -sig * xi, sig * xr);
  xr = h5 * (Or[2] * P[0] + Or[0] * P[2]); xi = h5 * (Oi[2] * P[0] + Oi[0] * P[2]);
  ACC(D_TJPR, xr, xi);
  ACC(D_TJPP, -sig * xi, sig * xr);
  xr = Or[1] * P[1] + Or[2] * P[2] + Or[3] * P[3]; xi = Oi[1] * P[1] + Oi[2] * P[2] + Oi[3] * P[3];
  ACC(D_TR, xr, xi);
  ACC(D_TP, -sig * xi, sig * xr);
  xr = h5 * (Or[0] * P[1] - Or[1] * P[0]); xi = h5 * (Oi[0] * P[1] - Oi[1] * P[0]);
  ACC(D_TJRR, -xi, xr);
  ACC(D_TJRP, -sig * xr, -sig * xi);
  xr = h5 * (Or[0] * P[3] - Or[3] * P[0]); xi = h5 * (Oi[0] * P[3] - Oi[3] * P[0]);
  ACC(D_TJZR, -xi, xr);
  ACC(D_TJZP, -sig * xr, -sig * xi);
}

// W_q(r, b) += sum over the staged rows a of phi_q(a, r) rho(a, b), q < NQ
template <class T, int NH, int NQ, int AK, int BWP>
__device__ __forceinline__ void dens_rows(const T* sphi, const T* srho, int na, int rl, int bl,
                                          T (&W)[NH][4][4][2]) {
  for (int aa = 0; aa < na; ++aa) {
    T f4[4];
    lds4(&sphi[(aa * DRT + rl) * 4], f4);
#pragma unroll
    for (int h = 0; h < NH; ++h) {
      T xr[4], xi[4];
      lds4(&srho[(0 * AK + aa) * BWP + 4 * bl + 32 * h], xr);
      lds4(&srho[(1 * AK + aa) * BWP + 4 * bl + 32 * h], xi);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          W[h][i][q][0] = fma(f4[q], xr[i], W[h][i][q][0]);
          W[h][i][q][1] = fma(f4[q], xi[i], W[h][i][q][1]);
        }
    }
  }
}

// grid (ceil(nghl/DRT), G, P*2 calls); block 256 = DRT mesh points x 8 column lanes.
// Thread (r, lane) owns mesh point r and columns b0 + 4*lane + i + 32*h of each chunk;
// W_q(r, b) = sum_a phi_q(a, r) rho_ab is accumulated over the rows of one spin, then
// folded into the thread's 28 complex densities, which are reduced over the 8 lanes
// at the end.  dpart: [P][2][G][2*ND][nghl]
template <class T>
__global__ void __launch_bounds__(256, sizeof(T) >= 8 ? 1 : 2) k_density(DevBasisT<T> B, DensCallT<T> c0, DensCallT<T> c1, int G,
                                                    T* __restrict__ dpart, const int* __restrict__ active) {
  constexpr int BT = DensTile<T>::BT, NH = BT / 4, BW = DensTile<T>::BW, BWP = DensTile<T>::BWP;
  constexpr int AK = DensTile<T>::AK;
  const int p = blockIdx.z >> 1, call = blockIdx.z & 1;
  if (!active[p]) return;
  const DensCallT<T>& C = call ? c1 : c0;
  const int g = blockIdx.y;
  const int r0 = blockIdx.x * DRT;
  const int rl = threadIdx.x >> 3, bl = threadIdx.x & 7;
  const int nghl = B.nghl;
  const int r = r0 + rl;
  const bool rok = r < nghl;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sphi = reinterpret_cast<T*>(smraw);   // [AK][DRT][4]
  T* srho = sphi + AK * DRT * 4;            // [2 pl][AK][BWP]
  const long long ps = (long long)B.dqp * nghl;
  T acc[2 * ND];
#pragma unroll
  for (int k = 0; k < 2 * ND; ++k) acc[k] = T(0);

  for (int kind = 0; kind < 2; ++kind) {  // 0: normal densities, 1: pairing densities
    const int* cols = kind == 0 ? C.rcols : C.kcols;
    const long long* offs = kind == 0 ? C.roffs : C.koffs;
    const T* base = kind == 0 ? C.rho : C.kap;
    const long long bsp = kind == 0 ? C.rho_sp : C.kap_sp, bspl = kind == 0 ? C.rho_spl : C.kap_spl;
    const int nq = kind == 0 ? 4 : 1;
    for (int ix = g; ix < B.nb; ix += G) {
      const int iy = cols[ix];
      if (iy < 0) continue;
      const int d = B.db[ix], dc = B.db[iy], nu = B.nup[ix];
      const int sa = B.st[ix], sb = B.st[iy];
      const T* mat = base + (long long)p * bsp + offs[ix];
      for (int b0 = 0; b0 < dc; b0 += BW) {
        // this thread's columns: spin (0 outside the block or the mesh) and phi_q(b, r),
        // loaded ahead of the row loop
        T sgb[NH][4], Pb[NH][4][4];
#pragma unroll
        for (int h = 0; h < NH; ++h)
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int b = b0 + 4 * bl + i + 32 * h;
            const bool ok = rok && b < dc;
            sgb[h][i] = ok ? (T)B.ns[sb + b] : T(0);
            const long long jb = sb + (ok ? b : 0);
#pragma unroll
            for (int q = 0; q < 4; ++q) Pb[h][i][q] = (ok && q < nq) ? B.phi[q * ps + jb * nghl + r] : T(0);
          }
        for (int s = 0; s < 2; ++s) {  // rows of spin up [0, nu), then spin down [nu, d)
          const int alo = s == 0 ? 0 : nu, ahi = s == 0 ? nu : d;
          if (alo >= ahi) continue;
          T W[NH][4][4][2];
#pragma unroll
          for (int h = 0; h < NH; ++h)
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int q = 0; q < 4; ++q) { W[h][i][q][0] = T(0); W[h][i][q][1] = T(0); }
          for (int a0 = alo; a0 < ahi; a0 += AK) {
            const int na = min(AK, ahi - a0);
            __syncthreads();
            for (int e = threadIdx.x; e < AK * DRT; e += blockDim.x) {
              const int rr = e % DRT, aa = e / DRT;
              T v[4] = {T(0), T(0), T(0), T(0)};
              if (aa < na && r0 + rr < nghl) {
#pragma unroll
                for (int q = 0; q < 4; ++q)
                  if (q < nq) v[q] = B.phi[q * ps + (long long)(sa + a0 + aa) * nghl + r0 + rr];
              }
              T* dst = &sphi[(aa * DRT + rr) * 4];
              dst[0] = v[0]; dst[1] = v[1]; dst[2] = v[2]; dst[3] = v[3];
            }
            // 8 consecutive rows x 4 columns per warp: coalesced reads, conflict-free writes
            for (int e = threadIdx.x; e < 2 * AK * BW; e += blockDim.x) {
              const int aa = (e & 7) + 8 * ((e >> 5) % (AK / 8));
              const int bb = ((e >> 3) & 3) + 4 * ((e >> 5) / (AK / 8) % (BW / 4));
              const int pl = e / (AK * BW);
              T v = T(0);
              if (aa < na && b0 + bb < dc) v = mat[(long long)pl * bspl + (a0 + aa) + (long long)(b0 + bb) * d];
              srho[(pl * AK + aa) * BWP + bb] = v;
            }
            __syncthreads();
            if (kind == 0) dens_rows<T, NH, 4, AK, BWP>(sphi, srho, na, rl, bl, W);
            else dens_rows<T, NH, 1, AK, BWP>(sphi, srho, na, rl, bl, W);
          }
          // fold the rows of spin s into the densities
          const T srow = s == 0 ? T(1) : T(-1);
#pragma unroll
          for (int h = 0; h < NH; ++h)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const T sg = sgb[h][i];
              if (sg == T(0)) continue;
              const T sig = sg < T(0) ? T(1) : T(-1);
              T Wr[4], Wi[4], Pq[4];
#pragma unroll
              for (int q = 0; q < 4; ++q) { Wr[q] = W[h][i][q][0]; Wi[q] = W[h][i][q][1]; Pq[q] = Pb[h][i][q]; }
              if (kind == 0) {
                if (sg == srow) dens_same(acc, Wr, Wi, Pq, sg);
                else dens_opp(acc, Wr, Wi, Pq, sig);
              } else {
                const T two = T(2);
                if (sg == srow) {
                  const T xr = two * Wr[0] * Pq[0], xi = two * Wi[0] * Pq[0];
                  ACC(D_SBR, sig * xr, sig * xi);
                  ACC(D_SBP, xi, -xr);
                } else {
                  const T xr = two * Wr[0] * Pq[0], xi = two * Wi[0] * Pq[0];
                  ACC(D_RB, -sg * xr, -sg * xi);
                  ACC(D_SBZ, xr, xi);
                }
              }
            }
        }
      }
    }
  }
#undef ACC
  // reduce over the 8 column lanes (same warp, low 3 bits of the lane)
#pragma unroll
  for (int k = 0; k < 2 * ND; ++k) {
    T v = acc[k];
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    acc[k] = v;
  }
  if (bl == 0 && rok) {
    T* out = dpart + (((long long)p * 2 + call) * G + g) * (2 * ND) * nghl;
#pragma unroll
    for (int k = 0; k < 2 * ND; ++k) out[(long long)k * nghl + r] = acc[k];
  }
}

// ---------------------------------------------------------------------------
// FP64 densities (the drop-in form and the anchors of the mixed form): a CTA of
// 32 mesh points x 8 column lanes; each lane accumulates W for one column b over
// chunks of DAK rows and folds it into its own 28 complex densities (registers),
// which are summed over the 8 lanes once, at the end.  FP64 is bound by the DFMA
// rate, so the tiles follow the blocks closely (8 columns per chunk, rows exact).
// ---------------------------------------------------------------------------
#define DBC 8    // b columns per chunk
#define DAK 16   // a rows per chunk

__device__ __forceinline__ double red8(double v) {
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  return v;
}

// grid (ceil(nghl/DRT), G, P*2 calls); block 256 = DRT r x DBC b
// dpart: [P][2][G][2*ND][nghl]
__global__ void __maxnreg__(192) k_density_fp64(DevBasis B, DensCall c0, DensCall c1, int G,
                                                      double* __restrict__ dpart, const int* __restrict__ active) {
  using T = double;
  const int p = blockIdx.z >> 1, call = blockIdx.z & 1;
  if (!active[p]) return;
  const DensCall& C = call ? c1 : c0;
  const int g = blockIdx.y;
  const int r0 = blockIdx.x * DRT;
  const int rl = threadIdx.x >> 3, bl = threadIdx.x & 7;
  const int nghl = B.nghl;
  const int r = r0 + rl;
  const bool rok = r < nghl;
  __shared__ T sphi[4][DAK][DRT];  // static smem: ~20 KB
  __shared__ T srho[2][DAK][DBC];
  T al[2 * ND];   // this lane's densities at mesh point r
#pragma unroll
  for (int k = 0; k < 2 * ND; ++k) al[k] = 0;
  const long long ps = (long long)B.dqp * nghl;
  const T h5 = (T)0.5, two = (T)2;

#define ACC(k, re, im) { al[2 * (k)] += (re); al[2 * (k) + 1] += (im); }

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
  T* out = dpart + (((long long)p * 2 + call) * G + g) * (2 * ND) * nghl;
#pragma unroll
  for (int k = 0; k < 2 * ND; ++k) {
    const T v = red8(al[k]);
    if (bl == 0 && rok) out[(long long)k * nghl + r] = v;
  }
}

// ---------------------------------------------------------------------------
// fold of W_q(r, b) = sum_a phi_q(a, r) rho_ab into the 28 local densities, one
// component q at a time (the terms of pnfam_hamiltonian_blas.f90:124-711 that
// contain W_q), for the tensor-core density kernel
// ---------------------------------------------------------------------------
// the terms of the density formulas that contain W_q of rows with the SAME spin as b
template <int Q>
__device__ __forceinline__ void fold_same(float (&acc)[2 * ND], float wr, float wi, const float (&P)[4], float sg) {
  const float h5 = 0.5f;
#define A_(k, re, im) { acc[2 * (k)] += (re); acc[2 * (k) + 1] += (im); }
  if (Q == 0) {
    A_(D_RHO, wr * P[0], wi * P[0]);
    A_(D_SZ, sg * wr * P[0], sg * wi * P[0]);
    A_(D_JP, h5 * wr * P[2], h5 * wi * P[2]);
    A_(D_TJPZ, sg * h5 * wr * P[2], sg * h5 * wi * P[2]);
    A_(D_JR, -h5 * wi * P[1], h5 * wr * P[1]);
    A_(D_TJRZ, -sg * h5 * wi * P[1], sg * h5 * wr * P[1]);
    A_(D_JZ, -h5 * wi * P[3], h5 * wr * P[3]);
    A_(D_TJZZ, -sg * h5 * wi * P[3], sg * h5 * wr * P[3]);
    A_(D_GS, sg * wr * P[3], sg * wi * P[3]);
  } else if (Q == 1) {
    A_(D_TAU, wr * P[1], wi * P[1]);
    A_(D_TZ, sg * wr * P[1], sg * wi * P[1]);
    A_(D_JR, h5 * wi * P[0], -h5 * wr * P[0]);
    A_(D_TJRZ, sg * h5 * wi * P[0], -sg * h5 * wr * P[0]);
    A_(D_FR, h5 * sg * wr * P[3], h5 * sg * wi * P[3]);
  } else if (Q == 2) {
    A_(D_JP, h5 * wr * P[0], h5 * wi * P[0]);
    A_(D_TJPZ, sg * h5 * wr * P[0], sg * h5 * wi * P[0]);
    A_(D_TAU, wr * P[2], wi * P[2]);
    A_(D_TZ, sg * wr * P[2], sg * wi * P[2]);
    A_(D_FP, -h5 * sg * wi * P[3], h5 * sg * wr * P[3]);
  } else {
    A_(D_TAU, wr * P[3], wi * P[3]);
    A_(D_TZ, sg * wr * P[3], sg * wi * P[3]);
    A_(D_JZ, h5 * wi * P[0], -h5 * wr * P[0]);
    A_(D_TJZZ, sg * h5 * wi * P[0], -sg * h5 * wr * P[0]);
    A_(D_GS, sg * wr * P[0], sg * wi * P[0]);
    A_(D_FR, h5 * sg * wr * P[1], h5 * sg * wi * P[1]);
    A_(D_FP, h5 * sg * wi * P[2], -h5 * sg * wr * P[2]);
    A_(D_FZ, sg * wr * P[3], sg * wi * P[3]);
  }
}

// the terms that contain W_q of rows with the OPPOSITE spin to b (sig = +1 if b is spin down)
template <int Q>
__device__ __forceinline__ void fold_opp(float (&acc)[2 * ND], float wr, float wi, const float (&P)[4], float sig) {
  const float h5 = 0.5f;
  if (Q == 0) {
    A_(D_GS, sig * wr * P[2] + wr * P[1], sig * wi * P[2] + wi * P[1]);
    A_(D_SR, wr * P[0], wi * P[0]);
    A_(D_SP, -sig * wi * P[0], sig * wr * P[0]);
    A_(D_TJPR, h5 * wr * P[2], h5 * wi * P[2]);
    A_(D_TJPP, -sig * h5 * wi * P[2], sig * h5 * wr * P[2]);
    A_(D_TJRR, -h5 * wi * P[1], h5 * wr * P[1]);
    A_(D_TJRP, -sig * h5 * wr * P[1], -sig * h5 * wi * P[1]);
    A_(D_TJZR, -h5 * wi * P[3], h5 * wr * P[3]);
    A_(D_TJZP, -sig * h5 * wr * P[3], -sig * h5 * wi * P[3]);
  } else if (Q == 1) {
    A_(D_GS, wr * P[0], wi * P[0]);
    A_(D_FR, wr * P[1] + sig * h5 * wr * P[2], wi * P[1] + sig * h5 * wi * P[2]);
    A_(D_FP, h5 * wi * P[2], -h5 * wr * P[2]);
    A_(D_FZ, h5 * wr * P[3], h5 * wi * P[3]);
    A_(D_TR, wr * P[1], wi * P[1]);
    A_(D_TP, -sig * wi * P[1], sig * wr * P[1]);
    A_(D_TJRR, h5 * wi * P[0], -h5 * wr * P[0]);
    A_(D_TJRP, sig * h5 * wr * P[0], sig * h5 * wi * P[0]);
  } else if (Q == 2) {
    A_(D_GS, -sig * wr * P[0], -sig * wi * P[0]);
    A_(D_FR, -sig * h5 * wr * P[1], -sig * h5 * wi * P[1]);
    A_(D_FP, -(sig * wi * P[2] + h5 * wi * P[1]), sig * wr * P[2] + h5 * wr * P[1]);
    A_(D_FZ, -sig * h5 * wr * P[3], -sig * h5 * wi * P[3]);
    A_(D_TJPR, h5 * wr * P[0], h5 * wi * P[0]);
    A_(D_TJPP, -sig * h5 * wi * P[0], sig * h5 * wr * P[0]);
    A_(D_TR, wr * P[2], wi * P[2]);
    A_(D_TP, -sig * wi * P[2], sig * wr * P[2]);
  } else {
    A_(D_FZ, h5 * (wr * P[1] + sig * wr * P[2]), h5 * (wi * P[1] + sig * wi * P[2]));
    A_(D_TR, wr * P[3], wi * P[3]);
    A_(D_TP, -sig * wi * P[3], sig * wr * P[3]);
    A_(D_TJZR, h5 * wi * P[0], -h5 * wr * P[0]);
    A_(D_TJZP, sig * h5 * wr * P[0], sig * h5 * wi * P[0]);
  }
}
#undef A_

struct DensTCArgs {
  const float* rho; long long rho_sp, rho_spl;   // as DensCallT, per call
  const int* rcols; const long long* roffs;
  const float* kap; long long kap_sp, kap_spl;
  const int* kcols; const long long* koffs;
};

// ---------------------------------------------------------------------------
// densities on the tensor cores with operands moved by the bulk-copy engine.
// A unit is (kind, block row ix, spin s of its rows, columns [b0, b0 + nc) of the
// block iy = cols[ix]), nc <= 64:
//   W[m][n] = sum_{a in s} phi_q(a, r) rho(a, b; pl),  m = q*32 + l (r = r0 + l),
//                                                     n = pl*nc + (b - b0)
// with K (the rows a of spin s) in chunks of 8.  Both operands are split into TF32
// high parts and remainders ahead of the kernel and laid out in the canonical
// K-major core-matrix order: A (phi) once per ground state for every (ix, s, chunk,
// 32-point mesh tile), B (rho of every active point) by k_dens_bsplit in each
// evaluation.  In the kernel one thread copies A and B chunks into a ring of
// DTC2_NS shared-memory stages (cp.async.bulk, completion on an mbarrier), one
// thread issues the 3xTF32 MMAs into one of two 128-column TMEM accumulators,
// and eight warps fold the finished accumulator (warp w: component q = w % 4, half
// of the columns; sums per row spin and column spin, turned into the 28 local
// densities at the end) while the other one fills.  dpart: [P][2][G][2*ND][nghl]
// ---------------------------------------------------------------------------
enum { DTC2_NS = 4, DTC2_FOLD = 256, DTC2_THREADS = DTC2_FOLD + 64, DTC2_MAXNC = 64 };
enum { DTC2_ACH = 2 * 128 * 8,                   // floats of one A chunk (hi, lo)
       DTC2_STAGE = DTC2_ACH + 2 * 128 * 8 };    // floats of one stage (A chunk, B chunk with npad <= 128)

struct DUnitTC {
  int kind, ix, iy, s;    // rows of block ix of spin s (0 up, 1 down), columns of block iy
  int b0, nc, npad, nk;   // columns [b0, b0 + nc), N = 2*nc padded to 16, K chunks of 8
  int achunk, nub;        // first A chunk of (ix, s); spin-up columns of block iy
  long long boff;         // floats: first B chunk of the unit within a point's B buffer
};
struct DBChunkTC {        // one B chunk: rows [a0, min(a0 + 8, ahi)) of a unit's columns
  int call, kind, ix, a0, ahi, b0, nc, npad;
  long long dst;          // floats within a point's B buffer
};
struct DAChunkTC { int ix, a0, ahi, pad_; };

__host__ __device__ constexpr size_t density_tc2_smem_bytes() {
  // the stage ring, then the column basis functions [64 b][32 r][4 q]; the
  // end-of-CTA reduction buffer [8 warps][2*ND][32] reuses the same memory
  return (size_t)(DTC2_NS * DTC2_STAGE + DTC2_MAXNC * 32 * 4) * sizeof(float);
}
static_assert(8 * 2 * ND * 32 <= DTC2_NS * DTC2_STAGE + DTC2_MAXNC * 32 * 4, "reduction buffer");

// A chunks (once per ground state): aphi[rt][chunk][hi | lo][128 x 8], rows m = q*32 + l
// grid (nachunk, ceil(nghl/32)), 256 threads
__global__ void __launch_bounds__(256) k_dens_asplit(DevBasisT<float> B, const DAChunkTC* __restrict__ chunks,
                                                     int nachunk, float* __restrict__ aphi) {
  const DAChunkTC ch = chunks[blockIdx.x];
  const int r0 = blockIdx.y * 32, nghl = B.nghl;
  const long long ps = (long long)B.dqp * nghl;
  float* dst = aphi + ((long long)blockIdx.y * nachunk + blockIdx.x) * DTC2_ACH;
  const int m = threadIdx.x & 127, k4 = threadIdx.x >> 7;
  const int q = m >> 5, r = r0 + (m & 31);
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  if (r < nghl) {
    const int a = ch.a0 + 4 * k4;
    const float* src = B.phi + q * ps + (long long)(B.st[ch.ix] + a) * nghl + r;
    if (a < ch.ahi) v.x = src[0];
    if (a + 1 < ch.ahi) v.y = src[nghl];
    if (a + 2 < ch.ahi) v.z = src[2 * nghl];
    if (a + 3 < ch.ahi) v.w = src[3 * nghl];
  }
  const int o = tc::cm_off(m, 4 * k4, 128);
  st_split4(dst + o, dst + 128 * 8 + o, v);
}

// B chunks of the listed points: bsplit[p][chunk.dst + (hi | lo)][npad x 8], rows n = pl*nc + b
// grid (nbchunk, nact), 256 threads
__global__ void __launch_bounds__(256) k_dens_bsplit(DevBasisT<float> B, DensTCArgs c0, DensTCArgs c1,
                                                     const DBChunkTC* __restrict__ chunks,
                                                     const int* __restrict__ actlist, float* __restrict__ bsplit,
                                                     long long bstride) {
  const DBChunkTC ch = chunks[blockIdx.x];
  const int p = actlist[blockIdx.y];
  const DensTCArgs& C = ch.call ? c1 : c0;
  const float* base = ch.kind == 0 ? C.rho : C.kap;
  const long long bsp = ch.kind == 0 ? C.rho_sp : C.kap_sp, bspl = ch.kind == 0 ? C.rho_spl : C.kap_spl;
  const long long off = (ch.kind == 0 ? C.roffs : C.koffs)[ch.ix];
  const float* mat = base + (long long)p * bsp + off;
  const int d = B.db[ch.ix];
  float* dst = bsplit + (long long)p * bstride + ch.dst;
  for (int e = threadIdx.x; e < 2 * ch.npad; e += blockDim.x) {
    const int n = e >> 1, k4 = e & 1;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (n < 2 * ch.nc) {
      const int pl = n >= ch.nc ? 1 : 0, b = n - pl * ch.nc;
      const int a = ch.a0 + 4 * k4;
      const float* src = mat + (long long)pl * bspl + (long long)(ch.b0 + b) * d + a;
      if (a < ch.ahi) v.x = src[0];
      if (a + 1 < ch.ahi) v.y = src[1];
      if (a + 2 < ch.ahi) v.z = src[2];
      if (a + 3 < ch.ahi) v.w = src[3];
    }
    const int o = tc::cm_off(n, 4 * k4, ch.npad);
    st_split4(dst + o, dst + ch.npad * 8 + o, v);
  }
}

// Every term of the density formulas is a fixed combination of the sums
//   T[s][up][q'] = sum over the columns b of spin up (1) or down (0) and the rows a
//                  of spin s of W_q(r, b) * phi_q'(b, r)   (re and im of W)
// so a fold warp accumulates only these sums per column (8 FMAs) and turns them
// into the 28 densities once, at the end (dtc2_densities).
// sum_unit: the columns [8*c8lo, 8*c8hi) of one unit (re of W at TMEM column b, im at
// nc + b); columns b < nupl are spin up.  KIND 1 (pairing): q' = 0 only.
template <int KIND, int NQ>
__device__ __forceinline__ void sum_unit(float (&T)[2][NQ][2], uint32_t lane_base, const float* sPb, int lane,
                                         int nc, int nupl, int c8lo, int c8hi, bool skip) {
  for (int c8 = c8lo; c8 < c8hi; ++c8) {
    float wre[8], wim[8];
    tc::tmem_ld8x2(lane_base + (uint32_t)(8 * c8), lane_base + (uint32_t)(nc + 8 * c8), wre, wim);
    if (skip) continue;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int b = 8 * c8 + i;
      if (b >= nc) break;
      const float4 pv = *reinterpret_cast<const float4*>(&sPb[(b * 32 + lane) * 4]);
      const float P[4] = {pv.x, pv.y, pv.z, pv.w};
      if (b < nupl) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          T[1][q][0] = fmaf(wre[i], P[q], T[1][q][0]);
          T[1][q][1] = fmaf(wim[i], P[q], T[1][q][1]);
        }
      } else {
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          T[0][q][0] = fmaf(wre[i], P[q], T[0][q][0]);
          T[0][q][1] = fmaf(wim[i], P[q], T[0][q][1]);
        }
      }
    }
  }
}

// the 28 densities of a fold warp of component Q from its sums: T0 (normal
// densities) and T1 (pairing densities, component 0) per row spin s and column spin
// up.  fold_same / fold_opp are linear in (wr, wi) * P, so a sum is folded as
// (wr, wi, P) = (1, 0, Re sums) plus (0, 1, Im sums).
template <int Q>
__device__ __forceinline__ void dtc2_densities(float (&acc)[2 * ND], const float (&T0)[2][2][4][2],
                                               const float (&T1)[2][2][1][2]) {
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int up = 0; up < 2; ++up) {
      const bool same = (up == 1) == (s == 0);
      const float sg = up ? 1.f : -1.f, sig = -sg;
      const float Pre[4] = {T0[s][up][0][0], T0[s][up][1][0], T0[s][up][2][0], T0[s][up][3][0]};
      const float Pim[4] = {T0[s][up][0][1], T0[s][up][1][1], T0[s][up][2][1], T0[s][up][3][1]};
      if (same) {
        fold_same<Q>(acc, 1.f, 0.f, Pre, sg);
        fold_same<Q>(acc, 0.f, 1.f, Pim, sg);
      } else {
        fold_opp<Q>(acc, 1.f, 0.f, Pre, sig);
        fold_opp<Q>(acc, 0.f, 1.f, Pim, sig);
      }
      if (Q == 0) {
        const float xr = 2.f * T1[s][up][0][0], xi = 2.f * T1[s][up][0][1];
        if (same) {
          acc[2 * D_SBR] += sig * xr; acc[2 * D_SBR + 1] += sig * xi;
          acc[2 * D_SBP] += xi; acc[2 * D_SBP + 1] += -xr;
        } else {
          acc[2 * D_RB] += -sg * xr; acc[2 * D_RB + 1] += -sg * xi;
          acc[2 * D_SBZ] += xr; acc[2 * D_SBZ + 1] += xi;
        }
      }
    }
}

// grid (ceil(nghl/32), G, 2*nact); DTC2_THREADS threads; dynamic smem density_tc2_smem_bytes().
// A CTA takes the units of its call with ix % G == g for its mesh tile and point.
__global__ void __launch_bounds__(DTC2_THREADS, 2) k_density_tc2(
    DevBasisT<float> B, const DUnitTC* __restrict__ units0, int nunit0, const DUnitTC* __restrict__ units1,
    int nunit1, const float* __restrict__ aphi, int nachunk, const float* __restrict__ bsplit, long long bstride,
    int G, const int* __restrict__ actlist, float* __restrict__ dpart, int* __restrict__ err) {
  const int p = actlist[blockIdx.z >> 1], call = blockIdx.z & 1;
  const DUnitTC* units = call ? units1 : units0;
  const int nunit = call ? nunit1 : nunit0;
  const int g = blockIdx.y, rt = blockIdx.x, r0 = rt * 32;
  const int nghl = B.nghl;
  const long long ps = (long long)B.dqp * nghl;
  extern __shared__ __align__(16) unsigned char smraw[];
  float* stages = reinterpret_cast<float*>(smraw);
  float* sPb = stages + DTC2_NS * DTC2_STAGE;
  __shared__ __align__(8) uint64_t full_bar[DTC2_NS], empty_bar[DTC2_NS], accf_bar[2], acce_bar[2];
  __shared__ uint32_t tslot;
  __shared__ volatile int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int i = 0; i < DTC2_NS; ++i) { tc::mbar_init(&full_bar[i], 1); tc::mbar_init(&empty_bar[i], 1); }
    for (int j = 0; j < 2; ++j) { tc::mbar_init(&accf_bar[j], 1); tc::mbar_init(&acce_bar[j], DTC2_FOLD); }
    abort_flag = 0;
  }
  if (warp == 0) tc::tmem_alloc(&tslot, 256);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tslot;
  const int q = warp & 3, half = warp >> 2;
  float T0[2][2][4][2], T1[2][2][1][2];   // fold warps: [row spin s][column spin up][q'][re, im]
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
#pragma unroll
        for (int k = 0; k < 4; ++k) T0[a][b][k][c] = 0.f;
        T1[a][b][0][c] = 0.f;
      }
  if (warp < DTC2_FOLD / 32) {
    // ---------------- fold warps ----------------
    int u = 0, skind = -1, siy = -1, sb0 = -1;
    for (int i = 0; i < nunit; ++i) {
      const DUnitTC U = units[i];
      if (U.ix % G != g) continue;
      const int j = u & 1;
      if (U.kind != skind || U.iy != siy || U.b0 != sb0) {
        // column basis functions of the unit's columns, once per column range
        asm volatile("bar.sync 1, %0;" ::"r"(DTC2_FOLD) : "memory");   // previous fold done with sPb
        const int sb = B.st[U.iy] + U.b0;
        for (int e = tid; e < U.nc * 32; e += DTC2_FOLD) {
          const int b = e >> 5, l = e & 31, r = r0 + l;
          float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
          if (r < nghl) {
            const float* src = B.phi + (long long)(sb + b) * nghl + r;
            v.x = src[0];
            if (U.kind == 0) { v.y = src[ps]; v.z = src[2 * ps]; v.w = src[3 * ps]; }
          }
          *reinterpret_cast<float4*>(&sPb[(b * 32 + l) * 4]) = v;
        }
        asm volatile("bar.sync 1, %0;" ::"r"(DTC2_FOLD) : "memory");
        skind = U.kind; siy = U.iy; sb0 = U.b0;
      }
      if (!abort_flag && !tc::mbar_wait(&accf_bar[j], (u >> 1) & 1)) abort_flag = 1;
      tc::fence_after();
      // pairing units: only the warps of component 0 read their rows
      if (U.kind == 0 || q == 0) {
        const int nb8 = (U.nc + 7) / 8;
        const int c8lo = half == 0 ? 0 : (nb8 + 1) / 2, c8hi = half == 0 ? (nb8 + 1) / 2 : nb8;
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(128 * j);
        const bool skip = abort_flag || r0 + lane >= nghl;
        const int nupl = U.nub - U.b0;
        if (U.kind == 0) {
          if (U.s == 0) sum_unit<0, 4>(T0[0], lane_base, sPb, lane, U.nc, nupl, c8lo, c8hi, skip);
          else sum_unit<0, 4>(T0[1], lane_base, sPb, lane, U.nc, nupl, c8lo, c8hi, skip);
        } else {
          if (U.s == 0) sum_unit<1, 1>(T1[0], lane_base, sPb, lane, U.nc, nupl, c8lo, c8hi, skip);
          else sum_unit<1, 1>(T1[1], lane_base, sPb, lane, U.nc, nupl, c8lo, c8hi, skip);
        }
      }
      tc::fence_before();
      tc::mbar_arrive(&acce_bar[j]);   // accumulator j free for the unit after next
      ++u;
    }
  } else if (tid == DTC2_FOLD) {
    // ---------------- MMA issuer ----------------
    int cc = 0, u = 0;
    for (int i = 0; i < nunit; ++i) {
      const DUnitTC U = units[i];
      if (U.ix % G != g) continue;
      const int j = u & 1;
      if (u >= 2 && !abort_flag && !tc::mbar_wait(&acce_bar[j], ((u >> 1) - 1) & 1)) abort_flag = 1;
      tc::fence_after();
      const uint32_t idesc = tc::idesc_tf32(128, U.npad);
      const uint32_t lboA = (128 / 8) * 128, lboB = (uint32_t)(U.npad / 8) * 128;
      const uint32_t acc_t = tmem + (uint32_t)(128 * j);
      for (int kc = 0; kc < U.nk; ++kc, ++cc) {
        const int st = cc % DTC2_NS;
        if (!abort_flag && !tc::mbar_wait(&full_bar[st], (cc / DTC2_NS) & 1)) abort_flag = 1;
        tc::fence_after();
        if (!abort_flag) {
          const float* sAh = stages + st * DTC2_STAGE;
          const float* sAl = sAh + 128 * 8;
          const float* sBh = sAh + DTC2_ACH;
          const float* sBl = sBh + U.npad * 8;
          const uint64_t ah = tc::sdesc(tc::smem_u32(sAh), lboA, 128);
          const uint64_t al = tc::sdesc(tc::smem_u32(sAl), lboA, 128);
          const uint64_t bh = tc::sdesc(tc::smem_u32(sBh), lboB, 128);
          const uint64_t bl = tc::sdesc(tc::smem_u32(sBl), lboB, 128);
          tc::mma_tf32(acc_t, ah, bh, idesc, kc > 0);
          tc::mma_tf32(acc_t, ah, bl, idesc, true);
          tc::mma_tf32(acc_t, al, bh, idesc, true);
        }
        tc::mma_commit(&empty_bar[st]);
      }
      tc::mma_commit(&accf_bar[j]);   // W of this unit complete
      ++u;
    }
    // nothing may be in flight when the tensor memory is released
    if (u > 0 && !tc::mbar_wait(&accf_bar[(u - 1) & 1], ((u - 1) >> 1) & 1)) abort_flag = 1;
  } else if (tid == DTC2_FOLD + 32) {
    // ---------------- bulk-copy producer ----------------
    const float* asrc = aphi + (long long)rt * nachunk * DTC2_ACH;
    const float* bsrc = bsplit + (long long)p * bstride;
    int cc = 0;   // chunks issued, in order
    for (int i = 0; i < nunit && !abort_flag; ++i) {
      const DUnitTC U = units[i];
      if (U.ix % G != g) continue;
      const uint32_t bbytes = (uint32_t)U.npad * 64;
      for (int kc = 0; kc < U.nk; ++kc) {
        const int st = cc % DTC2_NS;
        if (cc >= DTC2_NS && !abort_flag && !tc::mbar_wait(&empty_bar[st], ((cc / DTC2_NS) - 1) & 1)) abort_flag = 1;
        if (abort_flag) break;
        float* sA = stages + st * DTC2_STAGE;
        tc::mbar_expect_tx(&full_bar[st], (uint32_t)(DTC2_ACH * 4) + bbytes);
        tc::bulk_g2s(sA, asrc + (long long)(U.achunk + kc) * DTC2_ACH, DTC2_ACH * 4, &full_bar[st]);
        tc::bulk_g2s(sA + DTC2_ACH, bsrc + U.boff + (long long)kc * 16 * U.npad, bbytes, &full_bar[st]);
        ++cc;
      }
    }
    // no copy of this CTA may still be landing when the memory is reused: the last
    // DTC2_NS chunks issued are the only ones that can be in flight
    for (int k = cc > DTC2_NS ? cc - DTC2_NS : 0; k < cc; ++k)
      if (!tc::mbar_wait(&full_bar[k % DTC2_NS], (k / DTC2_NS) & 1)) abort_flag = 1;
  }
  // all folds done: each fold warp's densities from its sums, then the sum of the 8 warps
  tc::fence_before();
  const bool ok = __syncthreads_and(!abort_flag);
  float* red = stages;   // [8][2*ND][32]; the stages are no longer in use
  if (warp < 8) {
    float acc[2 * ND];
#pragma unroll
    for (int k = 0; k < 2 * ND; ++k) acc[k] = 0.f;
    switch (q) {
      case 0: dtc2_densities<0>(acc, T0, T1); break;
      case 1: dtc2_densities<1>(acc, T0, T1); break;
      case 2: dtc2_densities<2>(acc, T0, T1); break;
      default: dtc2_densities<3>(acc, T0, T1); break;
    }
#pragma unroll
    for (int k = 0; k < 2 * ND; ++k) red[(warp * 2 * ND + k) * 32 + lane] = acc[k];
  }
  __syncthreads();
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
  } else {
    float* out = dpart + (((long long)p * 2 + call) * G + g) * (2 * ND) * nghl;
    for (int e = tid; e < 2 * ND * 32; e += blockDim.x) {
      const int k = e / 32, l = e % 32;
      if (r0 + l >= nghl) continue;
      float v = 0.f;
#pragma unroll
      for (int w = 0; w < 8; ++w) v += red[(w * 2 * ND + k) * 32 + l];
      out[(long long)k * nghl + r0 + l] = v;
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tmem, 256);
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

// complex arithmetic of the mean field in the evaluation's precision S (FP64 for the
// FP64 form and the anchors, FP32 for the increment evaluations of the mixed form)
template <class S> struct cplxT { S r, i; };
template <class S> __device__ __forceinline__ cplxT<S> cmk(S r, S i) { cplxT<S> c; c.r = r; c.i = i; return c; }
template <class S> __device__ __forceinline__ cplxT<S> cadd(cplxT<S> a, cplxT<S> b) { return cmk<S>(a.r + b.r, a.i + b.i); }
template <class S> __device__ __forceinline__ cplxT<S> csc(S s, cplxT<S> a) { return cmk<S>(s * a.r, s * a.i); }

template <class T>
__global__ void __launch_bounds__(128) k_meanfield(DevBasisT<T> B, int G, const T* __restrict__ dpart,
                                                   T* __restrict__ mfout, const int* __restrict__ active) {
  using S = T;
  using C = cplxT<S>;
  const int p = blockIdx.y >> 1, call = blockIdx.y & 1;
  if (!active[p]) return;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int nghl = B.nghl;
  if (r >= nghl) return;
  C d[ND];
  const T* dp = dpart + ((long long)p * 2 + call) * G * (2 * ND) * nghl;
  const S wd = B.wdcori[r];
  for (int k = 0; k < ND; ++k) {
    S sr = S(0.0), si = S(0.0);
    for (int g = 0; g < G; ++g) {
      sr += (S)dp[((long long)g * 2 * ND + 2 * k) * nghl + r];
      si += (S)dp[((long long)g * 2 * ND + 2 * k + 1) * nghl + r];
    }
    d[k] = cmk<S>(sr * wd, si * wd);
  }
  const S crho = B.crho[r], cs = B.cs[r], cpair = B.cpair[r], cspair = B.cspair[r];
  const S cdrho = B.sc[0], ctau = B.sc[1], ctj0 = B.sc[2], ctj1 = B.sc[3], ctj2 = B.sc[4], crdj = B.sc[5];
  const S cds = B.sc[6], ct = B.sc[7], cj = B.sc[8], cgs = B.sc[9], cf = B.sc[10], csdj = B.sc[11];
  C mf[NMF];
  for (int k = 0; k < NMF; ++k) mf[k] = cmk<S>(S(0.0), S(0.0));
#define M_(iy, iz, sa, sb) mf[mfslot(iy, iz, sa, sb)]
#define ADD(iy, iz, sa, sb, sym, v) M_(iy, iz, sa, sb) = cadd<S>(M_(iy, iz, sa, sb), csc<S>(sym, v))
  const C rho = d[D_RHO], tau = d[D_TAU], tjrr = d[D_TJRR], tjpr = d[D_TJPR], tjzr = d[D_TJZR];
  const C tjrp = d[D_TJRP], tjpp = d[D_TJPP], tjzp = d[D_TJZP], tjrz = d[D_TJRZ], tjpz = d[D_TJPZ];
  const C tjzz = d[D_TJZZ], sr = d[D_SR], sp = d[D_SP], sz = d[D_SZ], tr = d[D_TR], tp = d[D_TP];
  const C tz = d[D_TZ], jr = d[D_JR], jp = d[D_JP], jz = d[D_JZ], fr = d[D_FR], fp = d[D_FP];
  const C fz = d[D_FZ], gs = d[D_GS];
  const C t0 = csc<S>(ctj0, cadd<S>(cadd<S>(tjrr, tjpp), tjzz));
  const C t1a = csc<S>(ctj1, cadd<S>(tjzr, csc<S>(-S(1.0), tjrz)));
  const C t1b = csc<S>(ctj1, cadd<S>(tjpz, csc<S>(-S(1.0), tjzp)));
  const C t2a = csc<S>(ctj2, cadd<S>(tjrz, tjzr));
  const C t2b = csc<S>(ctj2, cadd<S>(tjpz, tjzp));
  C aux;
  // diagonal in spin (pnfam_hamiltonian_blas.f90:783-905)
  M_(0, 0, 1, 1) = cadd<S>(csc<S>(S(2.0) * crho, rho), csc<S>(ctau, tau));
  M_(0, 0, -1, -1) = M_(0, 0, 1, 1);
  aux = cadd<S>(cadd<S>(csc<S>(S(2.0) * cs, sz), csc<S>(ct, tz)), csc<S>(cf, fz));
  ADD(0, 0, 1, 1, S(1.0), aux); ADD(0, 0, -1, -1, -S(1.0), aux);

  M_(0, 1, 1, 1) = csc<S>(-crdj, cadd<S>(tjpz, csc<S>(-S(1.0), tjzp)));
  M_(0, 1, -1, -1) = M_(0, 1, 1, 1);
  aux = csc<S>(-csdj, jp);
  ADD(0, 1, 1, 1, S(1.0), aux); ADD(0, 1, -1, -1, -S(1.0), aux);
  M_(1, 0, 1, 1) = M_(0, 1, 1, 1);
  M_(1, 0, -1, -1) = M_(0, 1, -1, -1);
  aux = cmk<S>(-t1a.i + S(0.5) * t2a.i, t1a.r - S(0.5) * t2a.r);
  ADD(0, 1, 1, 1, S(1.0), aux); ADD(0, 1, -1, -1, -S(1.0), aux);
  ADD(1, 0, 1, 1, -S(1.0), aux); ADD(1, 0, -1, -1, S(1.0), aux);
  aux = cmk<S>(cj * jr.i, -cj * jr.r);
  ADD(0, 1, 1, 1, S(1.0), aux); ADD(0, 1, -1, -1, S(1.0), aux);
  ADD(1, 0, 1, 1, -S(1.0), aux); ADD(1, 0, -1, -1, -S(1.0), aux);

  M_(0, 2, 1, 1) = csc<S>(cj, jp);
  M_(0, 2, -1, -1) = M_(0, 2, 1, 1);
  aux = cadd<S>(t1b, csc<S>(S(0.5), t2b));
  ADD(0, 2, 1, 1, S(1.0), aux); ADD(0, 2, -1, -1, -S(1.0), aux);
  M_(2, 0, 1, 1) = M_(0, 2, 1, 1);
  M_(2, 0, -1, -1) = M_(0, 2, -1, -1);
  aux = cmk<S>(-csdj * jr.i, csdj * jr.r);
  ADD(0, 2, 1, 1, S(1.0), aux); ADD(0, 2, -1, -1, -S(1.0), aux);
  ADD(2, 0, 1, 1, -S(1.0), aux); ADD(2, 0, -1, -1, S(1.0), aux);
  aux = cmk<S>(crdj * (tjzr.i - tjrz.i), -crdj * (tjzr.r - tjrz.r));
  ADD(0, 2, 1, 1, S(1.0), aux); ADD(0, 2, -1, -1, S(1.0), aux);
  ADD(2, 0, 1, 1, -S(1.0), aux); ADD(2, 0, -1, -1, -S(1.0), aux);

  M_(0, 3, 1, 1) = csc<S>(-crdj, cadd<S>(tjrp, csc<S>(-S(1.0), tjpr)));
  M_(0, 3, -1, -1) = M_(0, 3, 1, 1);
  aux = csc<S>(S(2.0) * cgs, gs);
  ADD(0, 3, 1, 1, S(1.0), aux); ADD(0, 3, -1, -1, -S(1.0), aux);
  M_(3, 0, 1, 1) = M_(0, 3, 1, 1);
  M_(3, 0, -1, -1) = M_(0, 3, -1, -1);
  aux = cmk<S>(t0.i - ctj2 * (tjrr.i + tjpp.i - S(2.0) * tjzz.i) / S(3.0),
            -t0.r + ctj2 * (tjrr.r + tjpp.r - S(2.0) * tjzz.r) / S(3.0));
  ADD(0, 3, 1, 1, S(1.0), aux); ADD(0, 3, -1, -1, -S(1.0), aux);
  ADD(3, 0, 1, 1, -S(1.0), aux); ADD(3, 0, -1, -1, S(1.0), aux);
  aux = cmk<S>(cj * jz.i, -cj * jz.r);
  ADD(0, 3, 1, 1, S(1.0), aux); ADD(0, 3, -1, -1, S(1.0), aux);
  ADD(3, 0, 1, 1, -S(1.0), aux); ADD(3, 0, -1, -1, -S(1.0), aux);

  M_(0, 4, 1, 1) = csc<S>(S(2.0) * cdrho, rho);
  M_(0, 4, -1, -1) = M_(0, 4, 1, 1);
  aux = csc<S>(S(2.0) * cds, sz);
  ADD(0, 4, 1, 1, S(1.0), aux); ADD(0, 4, -1, -1, -S(1.0), aux);
  M_(4, 0, 1, 1) = M_(0, 4, 1, 1);
  M_(4, 0, -1, -1) = M_(0, 4, -1, -1);

  M_(1, 2, 1, 1) = csc<S>(csdj, sz);
  M_(1, 2, -1, -1) = M_(1, 2, 1, 1);
  aux = csc<S>(crdj, rho);
  ADD(1, 2, 1, 1, S(1.0), aux); ADD(1, 2, -1, -1, -S(1.0), aux);
  M_(2, 1, 1, 1) = M_(1, 2, 1, 1);
  M_(2, 1, -1, -1) = M_(1, 2, -1, -1);

  M_(1, 3, 1, 1) = csc<S>(S(0.5) * cf, sr);
  M_(1, 3, -1, -1) = csc<S>(-S(1.0), M_(1, 3, 1, 1));
  M_(3, 1, 1, 1) = M_(1, 3, 1, 1);
  M_(3, 1, -1, -1) = M_(1, 3, -1, -1);
  aux = cmk<S>(-csdj * sp.i, csdj * sp.r);
  ADD(1, 3, 1, 1, S(1.0), aux); ADD(1, 3, -1, -1, S(1.0), aux);
  ADD(3, 1, 1, 1, -S(1.0), aux); ADD(3, 1, -1, -1, -S(1.0), aux);

  M_(2, 3, 1, 1) = csc<S>(-csdj, sr);
  M_(2, 3, -1, -1) = M_(2, 3, 1, 1);
  aux = cmk<S>(S(0.5) * cf * sp.i, -S(0.5) * cf * sp.r);
  ADD(2, 3, 1, 1, S(1.0), aux); ADD(2, 3, -1, -1, -S(1.0), aux);
  M_(3, 2, 1, 1) = M_(2, 3, -1, -1);
  M_(3, 2, -1, -1) = M_(2, 3, 1, 1);

  M_(1, 1, 1, 1) = csc<S>(S(4.0) * cdrho + ctau, rho);
  M_(1, 1, -1, -1) = M_(1, 1, 1, 1);
  aux = csc<S>(S(4.0) * cds + ct, sz);
  ADD(1, 1, 1, 1, S(1.0), aux); ADD(1, 1, -1, -1, -S(1.0), aux);
  M_(2, 2, 1, 1) = M_(1, 1, 1, 1);
  M_(2, 2, -1, -1) = M_(1, 1, -1, -1);
  M_(3, 3, 1, 1) = M_(1, 1, 1, 1);
  M_(3, 3, -1, -1) = M_(1, 1, -1, -1);
  aux = csc<S>(cf, sz);
  ADD(3, 3, 1, 1, S(1.0), aux); ADD(3, 3, -1, -1, -S(1.0), aux);

  // not diagonal in spin (pnfam_hamiltonian_blas.f90:908-1094)
  M_(0, 0, 1, -1) = cadd<S>(cadd<S>(csc<S>(S(2.0) * cs, sr), csc<S>(ct, tr)), csc<S>(cf, fr));
  M_(0, 0, -1, 1) = M_(0, 0, 1, -1);
  aux = cmk<S>(S(2.0) * cs * sp.i + ct * tp.i + cf * fp.i, -S(2.0) * cs * sp.r - ct * tp.r - cf * fp.r);
  ADD(0, 0, 1, -1, S(1.0), aux); ADD(0, 0, -1, 1, -S(1.0), aux);

  M_(0, 1, 1, -1) = csc<S>(S(2.0) * cgs, gs);
  M_(0, 1, -1, 1) = M_(0, 1, 1, -1);
  aux = cmk<S>(csdj * jz.i, -csdj * jz.r);
  ADD(0, 1, 1, -1, S(1.0), aux); ADD(0, 1, -1, 1, -S(1.0), aux);
  M_(1, 0, 1, -1) = M_(0, 1, 1, -1);
  M_(1, 0, -1, 1) = M_(0, 1, -1, 1);
  M_(0, 2, 1, -1) = M_(0, 1, 1, -1);
  M_(2, 0, -1, 1) = M_(1, 0, -1, 1);
  M_(2, 0, 1, -1) = csc<S>(-S(1.0), M_(0, 2, 1, -1));
  M_(0, 2, -1, 1) = csc<S>(-S(1.0), M_(2, 0, -1, 1));
  aux = csc<S>(-ctj1, cadd<S>(tjrp, csc<S>(-S(1.0), tjpr)));
  ADD(0, 1, 1, -1, S(1.0), aux); ADD(0, 1, -1, 1, -S(1.0), aux); ADD(1, 0, 1, -1, -S(1.0), aux); ADD(1, 0, -1, 1, S(1.0), aux);
  ADD(0, 2, 1, -1, S(1.0), aux); ADD(0, 2, -1, 1, S(1.0), aux); ADD(2, 0, 1, -1, S(1.0), aux); ADD(2, 0, -1, 1, S(1.0), aux);
  aux = cmk<S>(t0.i, -t0.r);
  ADD(0, 1, 1, -1, S(1.0), aux); ADD(0, 1, -1, 1, S(1.0), aux); ADD(1, 0, 1, -1, -S(1.0), aux); ADD(1, 0, -1, 1, -S(1.0), aux);
  ADD(0, 2, 1, -1, S(1.0), aux); ADD(0, 2, -1, 1, -S(1.0), aux); ADD(2, 0, 1, -1, S(1.0), aux); ADD(2, 0, -1, 1, -S(1.0), aux);
  aux = csc<S>(-S(0.5) * ctj2, cadd<S>(tjrp, tjpr));
  ADD(0, 1, 1, -1, S(1.0), aux); ADD(0, 1, -1, 1, -S(1.0), aux); ADD(1, 0, 1, -1, -S(1.0), aux); ADD(1, 0, -1, 1, S(1.0), aux);
  ADD(0, 2, 1, -1, -S(1.0), aux); ADD(0, 2, -1, 1, -S(1.0), aux); ADD(2, 0, 1, -1, -S(1.0), aux); ADD(2, 0, -1, 1, -S(1.0), aux);
  aux = cmk<S>(-ctj2 * (-S(2.0) * tjrr.i + tjpp.i + tjzz.i) / S(3.0), ctj2 * (-S(2.0) * tjrr.r + tjpp.r + tjzz.r) / S(3.0));
  ADD(0, 1, 1, -1, S(1.0), aux); ADD(0, 1, -1, 1, S(1.0), aux); ADD(1, 0, 1, -1, -S(1.0), aux); ADD(1, 0, -1, 1, -S(1.0), aux);
  aux = cmk<S>(-ctj2 * (tjrr.i - S(2.0) * tjpp.i + tjzz.i) / S(3.0), ctj2 * (tjrr.r - S(2.0) * tjpp.r + tjzz.r) / S(3.0));
  ADD(0, 2, 1, -1, S(1.0), aux); ADD(0, 2, -1, 1, -S(1.0), aux); ADD(2, 0, 1, -1, S(1.0), aux); ADD(2, 0, -1, 1, -S(1.0), aux);

  M_(0, 3, 1, -1) = csc<S>(csdj, jp);
  M_(0, 3, -1, 1) = M_(0, 3, 1, -1);
  aux = cmk<S>(-csdj * jr.i, csdj * jr.r);
  ADD(0, 3, 1, -1, S(1.0), aux); ADD(0, 3, -1, 1, -S(1.0), aux);
  M_(3, 0, 1, -1) = M_(0, 3, 1, -1);
  M_(3, 0, -1, 1) = M_(0, 3, -1, 1);
  aux = cmk<S>(t1a.i + S(0.5) * t2a.i, -t1a.r - S(0.5) * t2a.r);
  ADD(0, 3, 1, -1, S(1.0), aux); ADD(0, 3, -1, 1, S(1.0), aux); ADD(3, 0, 1, -1, -S(1.0), aux); ADD(3, 0, -1, 1, -S(1.0), aux);
  aux = cadd<S>(t1b, csc<S>(-S(0.5), t2b));
  ADD(0, 3, 1, -1, S(1.0), aux); ADD(0, 3, -1, 1, -S(1.0), aux); ADD(3, 0, 1, -1, -S(1.0), aux); ADD(3, 0, -1, 1, S(1.0), aux);

  M_(0, 4, 1, -1) = csc<S>(S(2.0) * cds, sr);
  M_(0, 4, -1, 1) = M_(0, 4, 1, -1);
  aux = cmk<S>(S(2.0) * cds * sp.i, -S(2.0) * cds * sp.r);
  ADD(0, 4, 1, -1, S(1.0), aux); ADD(0, 4, -1, 1, -S(1.0), aux);
  M_(4, 0, 1, -1) = M_(0, 4, 1, -1);
  M_(4, 0, -1, 1) = M_(0, 4, -1, 1);

  M_(1, 2, 1, -1) = cmk<S>(-S(0.5) * cf * sp.i, S(0.5) * cf * sp.r);
  M_(1, 2, -1, 1) = M_(1, 2, 1, -1);
  aux = csc<S>(S(0.5) * cf, sr);
  ADD(1, 2, 1, -1, S(1.0), aux); ADD(1, 2, -1, 1, -S(1.0), aux);
  M_(2, 1, 1, -1) = csc<S>(-S(1.0), M_(1, 2, 1, -1));
  M_(2, 1, -1, 1) = csc<S>(-S(1.0), M_(1, 2, -1, 1));

  M_(1, 3, 1, -1) = csc<S>(S(0.5) * cf, sz);
  M_(1, 3, -1, 1) = M_(1, 3, 1, -1);
  aux = csc<S>(crdj, rho);
  ADD(1, 3, 1, -1, S(1.0), aux); ADD(1, 3, -1, 1, -S(1.0), aux);
  M_(3, 1, 1, -1) = M_(1, 3, -1, 1);
  M_(3, 1, -1, 1) = M_(1, 3, 1, -1);
  M_(3, 2, 1, -1) = M_(3, 1, 1, -1);
  M_(2, 3, -1, 1) = M_(1, 3, -1, 1);
  M_(2, 3, 1, -1) = csc<S>(-S(1.0), M_(1, 3, 1, -1));
  M_(3, 2, -1, 1) = csc<S>(-S(1.0), M_(3, 1, -1, 1));

  M_(3, 3, 1, -1) = csc<S>(ct + S(4.0) * cds, sr);
  M_(3, 3, -1, 1) = M_(3, 3, 1, -1);
  aux = cmk<S>((ct + S(4.0) * cds) * sp.i, -(ct + S(4.0) * cds) * sp.r);
  ADD(3, 3, 1, -1, S(1.0), aux); ADD(3, 3, -1, 1, -S(1.0), aux);
  M_(1, 1, 1, -1) = M_(3, 3, 1, -1);
  M_(1, 1, -1, 1) = M_(3, 3, -1, 1);
  aux = csc<S>(cf, sr);
  ADD(1, 1, 1, -1, S(1.0), aux); ADD(1, 1, -1, 1, S(1.0), aux);
  M_(2, 2, 1, -1) = M_(3, 3, 1, -1);
  M_(2, 2, -1, 1) = M_(3, 3, -1, 1);
  aux = cmk<S>(cf * sp.i, -cf * sp.r);
  ADD(2, 2, 1, -1, S(1.0), aux); ADD(2, 2, -1, 1, -S(1.0), aux);
#undef ADD
#undef M_
  // pairing fields (pnfam_hamiltonian_blas.f90:1201-1208): index (sa, sb)
  const C rb = d[D_RB], sbr = d[D_SBR], sbp = d[D_SBP], sbz = d[D_SBZ];
  mf[100] = cmk<S>(cspair * (sbr.r + sbp.i), cspair * (sbr.i - sbp.r));        // a+ b+
  mf[101] = cmk<S>(cpair * rb.r - cspair * sbz.r, cpair * rb.i - cspair * sbz.i); // a+ b-
  mf[102] = cmk<S>(-cpair * rb.r - cspair * sbz.r, -cpair * rb.i - cspair * sbz.i); // a- b+
  mf[103] = cmk<S>(cspair * (-sbr.r + sbp.i), cspair * (-sbr.i - sbp.r));      // a- b-
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
  int a0, na;      // row tile inside block ix (spin-uniform), na <= 1024 / tn
  int b0, nbc;     // column tile inside block iy, nbc <= tn
  int sa;          // spin of the rows (+1/-1)
  int mode;        // 0: mean field (5 components), 1: pairing (1 component)
  int call;        // 0: pn, 1: np
  int outq;        // HSP quadrant 0..3 (m11, m12, m21, m22)
  int tn, pad_;    // tile shape: (1024 / tn) rows x tn columns, tn = 32, 16 or 8
  long long ooff;  // block offset inside the quadrant
};

#define HRC 16   // mesh points per K chunk

// FP64 field projection: output tiles of TM = 1024 / TN rows x TN columns (TN = 32, 16
// or 8, chosen per block pair from the block sizes so that little of the FP64 pipe goes
// to padding), 2 x 2 outputs per thread; warps whose rows lie beyond the tile's na skip
// the FMAs (the DFMA rate is the bound).  grid (ntasks, P); 256 threads; dynamic smem
// hproj_fp64_smem_bytes()
// mesh points per K chunk of a shape: 16, or 8 for the 128-row tiles, so that every
// shape stays within the 94.7 KB of the 32 x 32 tiles and a CTA of the FP32 kernels
// (pair-tensor GEMM: 128 KB) still fits beside one on an SM
__host__ __device__ constexpr int hproj_fp64_hr(int tn) { return tn == 8 ? 8 : HRC; }
__host__ __device__ constexpr size_t hproj_fp64_smem_tn(int tn) {
  return (size_t)(5 * (1024 / tn) + 5 * tn + 25 * 4 + 5 * tn * 2) * hproj_fp64_hr(tn) * sizeof(double);
}
__host__ __device__ constexpr size_t hproj_fp64_smem_bytes() {
  return hproj_fp64_smem_tn(8) > hproj_fp64_smem_tn(32) ? hproj_fp64_smem_tn(8) : hproj_fp64_smem_tn(32);
}

template <int TN, int HR>
__device__ __forceinline__ void hproj_fp64_tile(const DevBasis& B, const HTask& Th, const double* __restrict__ mfp,
                                                double* __restrict__ hsp, long long nxy, int p,
                                                unsigned char* smraw, signed char* sns) {
  using T = double;
  constexpr int TM = 1024 / TN, TX = TN / 2;
  const int nghl = B.nghl;
  const long long ps = (long long)B.dqp * nghl;
  const int nc = Th.mode == 0 ? 5 : 1;
  T* sA = reinterpret_cast<T*>(smraw);     // [5][TM][HR]
  T* sPb = sA + 5 * TM * HR;               // [5][TN][HR]
  T* sMF = sPb + 5 * TN * HR;              // [25][2 sb][2 re/im][HR]
  T* sH = sMF + 25 * 2 * 2 * HR;           // [5][TN][2][HR]
  const int ja0 = B.st[Th.ix] + Th.a0, jb0 = B.st[Th.iy] + Th.b0;
  if (threadIdx.x < TN) sns[threadIdx.x] = threadIdx.x < Th.nbc ? B.ns[jb0 + threadIdx.x] : (signed char)1;
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  // rows 2 ty, 2 ty + 1; the rows of warp w start at 64 w / TX
  const bool rows_live = (64 * (int)(threadIdx.x >> 5)) / TX < Th.na;
  T ar[2][2] = {{0, 0}, {0, 0}}, ai[2][2] = {{0, 0}, {0, 0}};
  for (int r0 = 0; r0 < nghl; r0 += HR) {
    const int nr = min(HR, nghl - r0);
    __syncthreads();
    for (int e = threadIdx.x; e < nc * TM * HR; e += 256) {
      const int q = e / (TM * HR), rem = e % (TM * HR), aa = rem / HR, rr = rem % HR;
      T va = 0;
      if (rr < nr && aa < Th.na) va = B.phi[q * ps + (long long)(ja0 + aa) * nghl + r0 + rr];
      sA[(q * TM + aa) * HR + rr] = va;
    }
    for (int e = threadIdx.x; e < nc * TN * HR; e += 256) {
      const int q = e / (TN * HR), rem = e % (TN * HR), bb = rem / HR, rr = rem % HR;
      T vb = 0;
      if (rr < nr && bb < Th.nbc) vb = B.phi[q * ps + (long long)(jb0 + bb) * nghl + r0 + rr];
      sPb[(q * TN + bb) * HR + rr] = vb;
    }
    if (Th.mode == 0) {
      for (int e = threadIdx.x; e < 25 * 2 * 2 * HR; e += 256) {
        const int pair = e / (4 * HR), rem = e % (4 * HR), sb = rem / (2 * HR), rem2 = rem % (2 * HR);
        const int ri = rem2 / HR, rr = rem2 % HR;
        const int iy = pair / 5, iz = pair % 5;
        T v = 0;
        if (rr < nr) v = mfp[((long long)mfslot(iy, iz, Th.sa, sb == 0 ? 1 : -1) * 2 + ri) * nghl + r0 + rr];
        sMF[e] = v;
      }
    } else {
      for (int e = threadIdx.x; e < 2 * 2 * HR; e += 256) {
        const int sb = e / (2 * HR), rem = e % (2 * HR), ri = rem / HR, rr = rem % HR;
        const int slot = 100 + (Th.sa < 0 ? 2 : 0) + sb;
        sMF[e] = rr < nr ? mfp[((long long)slot * 2 + ri) * nghl + r0 + rr] : (T)0;
      }
    }
    __syncthreads();
    // hpsi(iy, b, r) = sum_iz mf(iy, iz, sa, s_b)(r) phi_iz(b, r), for the tile's live columns
    for (int e = threadIdx.x; e < nc * TN * HR; e += 256) {
      const int iy = e / (TN * HR), rem = e % (TN * HR), bb = rem / HR, rr = rem % HR;
      T hr = 0, hi = 0;
      if (bb < Th.nbc) {
        const int sb = sns[bb] > 0 ? 0 : 1;
        if (Th.mode == 0) {
#pragma unroll
          for (int iz = 0; iz < 5; ++iz) {
            const T f = sPb[(iz * TN + bb) * HR + rr];
            const T* m = &sMF[((iy * 5 + iz) * 4 + sb * 2) * HR];
            hr = fma(m[rr], f, hr); hi = fma(m[HR + rr], f, hi);
          }
        } else {
          const T f = sPb[bb * HR + rr];
          hr = sMF[(sb * 2) * HR + rr] * f; hi = sMF[(sb * 2 + 1) * HR + rr] * f;
        }
      }
      sH[((iy * TN + bb) * 2) * HR + rr] = hr;
      sH[((iy * TN + bb) * 2 + 1) * HR + rr] = hi;
    }
    __syncthreads();
    if (rows_live)
    for (int q = 0; q < nc; ++q) {
      for (int rr = 0; rr < HR; ++rr) {
        const T a0 = sA[(q * TM + ty * 2) * HR + rr], a1 = sA[(q * TM + ty * 2 + 1) * HR + rr];
        const T h0r = sH[((q * TN + tx * 2) * 2) * HR + rr], h0i = sH[((q * TN + tx * 2) * 2 + 1) * HR + rr];
        const T h1r = sH[((q * TN + tx * 2 + 1) * 2) * HR + rr], h1i = sH[((q * TN + tx * 2 + 1) * 2 + 1) * HR + rr];
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

__global__ void __launch_bounds__(256) k_hproj_fp64(DevBasis B, const HTask* __restrict__ tasks,
                                                    const double* __restrict__ mf, double* __restrict__ hsp,
                                                    long long nxy, const int* __restrict__ active) {
  const int p = blockIdx.y;
  if (!active[p]) return;
  const HTask Th = tasks[blockIdx.x];
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ signed char sns[32];
  const double* mfp = mf + ((long long)p * 2 + Th.call) * NMF * 2 * B.nghl;
  if (Th.tn == 8) hproj_fp64_tile<8, hproj_fp64_hr(8)>(B, Th, mfp, hsp, nxy, p, smraw, sns);
  else if (Th.tn == 16) hproj_fp64_tile<16, hproj_fp64_hr(16)>(B, Th, mfp, hsp, nxy, p, smraw, sns);
  else hproj_fp64_tile<32, hproj_fp64_hr(32)>(B, Th, mfp, hsp, nxy, p, smraw, sns);
}

// ---------------------------------------------------------------------------
// field projection on the tensor cores (FP32 data, 3xTF32 products).
// One CTA computes, for one (block pair, spin segment of the rows) and up to pg
// points, D[m][n] = sum_k hpsi[k][m] phi[k][n] with
//   m = pl*64 + j, j = (point in the group)*nbc + b   (rows: Re, then Im of hpsi)
//   n = a (the rows of the output block, N padded to np)
//   k = (q, r), 32 mesh points of one component q per chunk.
// Warps 0-7 produce the A operand of a chunk (hpsi generated from the field
// tensor and the column basis functions) into one of two shared-memory stages;
// the B operand (the row basis functions, constant: split into TF32 hi and lo once
// per operator in the canonical layout) is copied in by the bulk-copy engine.
// Warp 8 issues the MMAs of a chunk as soon as its stage is full and releases the
// stage through tcgen05.commit, so operand production and tensor-core work
// overlap.  D accumulates in tensor memory and out_ab = 2 D.
// ---------------------------------------------------------------------------
struct HTaskTC {
  int ix, iy, a0, na, b0, nbc, sa, mode, call, outq;
  int np;          // N of the MMA: na rounded up to 16
  int pg;          // points per CTA (pg * nbc <= 64)
  long long ooff;
  long long tphi;  // floats: the pre-split row basis functions of rows a0..a0+na of block ix
};
enum { HTC_K = 32, HTC_MAXB = 64, HTC_MAXN = 128, HTC_MAXPG = 8, HTC_PROD = 256, HTC_THREADS = HTC_PROD + 32 };
// pre-split B operand of one row tile (rows a0..a0+na of block ix): for component q
// and mesh chunk rc (32 points), [hi | lo][np x 32] at off + (q * nrc + rc) * 64 * np
struct HPTile { int ix, a0, na, np; long long off; };

// grid (ntiles, 5 * nrc), 256 threads
__global__ void __launch_bounds__(256) k_hproj_bsplit(DevBasisT<float> B, const HPTile* __restrict__ tiles, int nrc,
                                                      float* __restrict__ hphi) {
  const HPTile t = tiles[blockIdx.x];
  const int q = blockIdx.y / nrc, r0 = (blockIdx.y % nrc) * HTC_K;
  const int nghl = B.nghl;
  const long long ps = (long long)B.dqp * nghl;
  float* dst = hphi + t.off + (long long)blockIdx.y * 64 * t.np;
  const int ja0 = B.st[t.ix] + t.a0;
  for (int e = threadIdx.x; e < t.np * 8; e += blockDim.x) {
    const int n = e % t.np, r4 = e / t.np;
    const float4 v = ld_row4(B.phi + q * ps + (long long)(ja0 + n) * nghl, r0 + 4 * r4, nghl, n < t.na);
    const int o = tc::cm_off(n, 4 * r4, t.np);
    st_split4(dst + o, dst + 32 * t.np + o, v);
  }
}

// dynamic shared memory for tiles of at most npmax output rows: two stages of
// A (128 x 32, hi and lo) and B (npmax x 32, hi and lo), then the field tensor
// of the current chunk [pg][2 sb][5 iz][2 re/im][32 r]
__host__ __device__ constexpr size_t hproj_tc_smem_bytes(int npmax) {
  return (size_t)(2 * (2 * 128 * HTC_K + 2 * npmax * HTC_K) + HTC_MAXPG * 2 * 5 * 2 * HTC_K) * sizeof(float);
}

// grid (ntasks, point groups); HTC_THREADS threads; dynamic smem hproj_tc_smem_bytes(npmax)
// actlist[nact]: the points to evaluate; err: set to 1 if a wait on the tensor
// cores gave up (the CTA then writes nothing)
__global__ void __launch_bounds__(HTC_THREADS, 2) k_hproj_tc(DevBasisT<float> B, const HTaskTC* __restrict__ tasks,
                                                             const int* __restrict__ actlist, int nact, int npmax,
                                                             const float* __restrict__ mf,
                                                             const float* __restrict__ hphi, float* __restrict__ hsp,
                                                             long long nxy, int* __restrict__ err) {
  const HTaskTC Th = tasks[blockIdx.x];
  const int g0 = blockIdx.y * Th.pg;
  if (g0 >= nact) return;
  const int npg = min(Th.pg, nact - g0);
  extern __shared__ __align__(16) unsigned char smraw[];
  float* stage_base = reinterpret_cast<float*>(smraw);
  const int stage_floats = 2 * 128 * HTC_K + 2 * npmax * HTC_K;
  float* sMF = stage_base + 2 * stage_floats;   // [pg][2 sb][5 iz][2 re/im][32 r]
  __shared__ __align__(8) uint64_t full_bar[2], empty_bar[2];
  __shared__ uint32_t tslot;
  __shared__ volatile int abort_flag;
  __shared__ signed char sns[HTC_MAXB];
  __shared__ int spt[HTC_MAXPG];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int nbc = Th.nbc, NP = Th.np, nj = npg * nbc;
  const int nghl = B.nghl;
  const long long ps = (long long)B.dqp * nghl;
  const int jb0 = B.st[Th.iy] + Th.b0;
  const int nc = Th.mode == 0 ? 5 : 1;
  const int nrc = (nghl + HTC_K - 1) / HTC_K;   // chunks per component
  const int nchunk = nc * nrc;
  const uint32_t ncols = NP <= 32 ? 32u : NP <= 64 ? 64u : NP <= 128 ? 128u : 256u;
  if (tid < HTC_MAXB) sns[tid] = tid < nbc ? B.ns[jb0 + tid] : (signed char)1;
  if (tid < HTC_MAXPG) spt[tid] = tid < npg ? actlist[g0 + tid] : 0;
  if (tid == 0) {
    tc::mbar_init(&full_bar[0], HTC_PROD); tc::mbar_init(&full_bar[1], HTC_PROD);
    tc::mbar_init(&empty_bar[0], 1); tc::mbar_init(&empty_bar[1], 1);
    abort_flag = 0;
  }
  if (warp == 0) tc::tmem_alloc(&tslot, ncols);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tslot;
  const float* mfbase = mf + (long long)Th.call * NMF * 2 * nghl;
  if (warp < HTC_PROD / 32) {
    // ---------------- producers ----------------
    // chunks in mesh-point-major order: the column basis functions phi_iz(b, r) of a
    // thread's two A items stay in registers for the nc components of one r range.
    // Everything that does not depend on the chunk is computed once: the hpsi row
    // (point, column), spin and shared-memory offsets of the two A items.
    float4 fz[2][5];
    int a_m[2], a_row[2], a_ore[2], a_oim[2];   // a_row < 0: no hpsi row
#pragma unroll
    for (int it = 0; it < 2; ++it) {
      const int e = tid + it * HTC_PROD;
      const int j = e % HTC_MAXB, r4 = e / HTC_MAXB;
      const int pi = j < nj ? j / nbc : 0, b = j < nj ? j % nbc : 0;
      const int sbi = sns[b] > 0 ? 0 : 1;
      a_m[it] = (((pi * 2 + sbi) * 5) * 2) * HTC_K + 4 * r4;
      a_row[it] = j < nj ? jb0 + b : -1;
      a_ore[it] = tc::cm_off(j, 4 * r4, 128);
      a_oim[it] = tc::cm_off(64 + j, 4 * r4, 128);
    }
    int lc0 = -1, lc1 = -1;   // thread 0: last chunk copied into stage 0, stage 1
    for (int c = 0; c < nchunk; ++c) {
      const int st = c & 1;
      if (c >= 2 && !abort_flag && !tc::mbar_wait(&empty_bar[st], ((c >> 1) - 1) & 1)) abort_flag = 1;
      float* sAh = stage_base + st * stage_floats;
      float* sAl = sAh + 128 * HTC_K;
      float* sBh = sAl + 128 * HTC_K;
      const int q = c % nc, r0 = (c / nc) * HTC_K;
      bool issued = false;
      if (tid == 0 && !abort_flag) {
        // B: the row basis functions phi_q(a, r) of this chunk, pre-split (hi then lo,
        // NP x 32 each); this thread's arrival on the stage comes with the copy
        const uint32_t bbytes = (uint32_t)NP * HTC_K * 2 * 4;
        tc::mbar_expect_tx(&full_bar[st], bbytes);
        tc::bulk_g2s(sBh, hphi + Th.tphi + (long long)(q * nrc + c / nc) * 64 * NP, bbytes, &full_bar[st]);
        issued = true;
        if (st == 0) lc0 = c; else lc1 = c;
      }
      // the field tensor of this chunk (component q, mesh points r0..r0+31) of every
      // point of the group, shared by all rows; the barriers keep one chunk's copy
      // from being overwritten while another chunk's rows are generated
      asm volatile("bar.sync 1, %0;" ::"r"(HTC_PROD) : "memory");
      for (int e = tid; e < npg * 2 * 5 * 2 * 8; e += HTC_PROD) {
        const int r4 = e & 7, ri = (e >> 3) & 1, iz = (e >> 4) % 5, sbi = (e / 80) & 1, pi = e / 160;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (iz < nc) {
          const int sb = sbi == 0 ? 1 : -1;
          const int slot = Th.mode == 0 ? mfslot(q, iz, Th.sa, sb) : 100 + (Th.sa < 0 ? 2 : 0) + sbi;
          const float* mp = mfbase + (long long)spt[pi] * 2 * NMF * 2 * nghl;
          v = ld_row4(mp + ((long long)slot * 2 + ri) * nghl, r0 + 4 * r4, nghl, true);
        }
        *reinterpret_cast<float4*>(&sMF[((((pi * 2 + sbi) * 5 + iz) * 2 + ri) * HTC_K) + 4 * r4]) = v;
      }
      asm volatile("bar.sync 1, %0;" ::"r"(HTC_PROD) : "memory");
      if (!abort_flag) {
        // A: hpsi rows, Re at j, Im at 64 + j, four mesh points per item
#pragma unroll
        for (int it = 0; it < 2; ++it) {
          const int r = r0 + 4 * ((tid + it * HTC_PROD) / HTC_MAXB);
          float4 hr = make_float4(0.f, 0.f, 0.f, 0.f), hi = hr;
          if (a_row[it] >= 0) {
            if (q == 0) {
#pragma unroll
              for (int iz = 0; iz < 5; ++iz)
                if (iz < nc) fz[it][iz] = ld_row4(B.phi + iz * ps + (long long)a_row[it] * nghl, r, nghl, true);
            }
            const float* m = &sMF[a_m[it]];
#pragma unroll
            for (int iz = 0; iz < 5; ++iz)
              if (iz < nc) {
                fma4(hr, *reinterpret_cast<const float4*>(m + (iz * 2 + 0) * HTC_K), fz[it][iz]);
                fma4(hi, *reinterpret_cast<const float4*>(m + (iz * 2 + 1) * HTC_K), fz[it][iz]);
              }
          }
          st_split4(sAh + a_ore[it], sAl + a_ore[it], hr);
          st_split4(sAh + a_oim[it], sAl + a_oim[it], hi);
        }
      }
      tc::fence_async_smem();
      if (!issued) tc::mbar_arrive(&full_bar[st]);
    }
    // no copy may still be landing when the memory is reused (the last two chunks
    // are the only ones that can be in flight)
    if (tid == 0) {
      if (lc0 >= 0 && !tc::mbar_wait(&full_bar[0], (lc0 >> 1) & 1)) abort_flag = 1;
      if (lc1 >= 0 && !tc::mbar_wait(&full_bar[1], (lc1 >> 1) & 1)) abort_flag = 1;
    }
  } else if (tid == HTC_PROD) {
    // ---------------- MMA issuer (one thread of warp 8) ----------------
    const uint32_t idesc = tc::idesc_tf32(128, NP);
    const uint32_t lboA = (128 / 8) * 128, lboB = (uint32_t)(NP / 8) * 128;
    for (int c = 0; c < nchunk; ++c) {
      const int st = c & 1;
      if (!abort_flag && !tc::mbar_wait(&full_bar[st], (c >> 1) & 1)) abort_flag = 1;
      tc::fence_after();
      if (!abort_flag) {
        const float* sAh = stage_base + st * stage_floats;
        const float* sAl = sAh + 128 * HTC_K;
        const float* sBh = sAl + 128 * HTC_K;
        const float* sBl = sBh + NP * HTC_K;
#pragma unroll
        for (int ks = 0; ks < HTC_K / 8; ++ks) {
          const uint32_t oa = ks * 2 * lboA, ob = ks * 2 * lboB;
          const uint64_t ah = tc::sdesc(tc::smem_u32(sAh) + oa, lboA, 128);
          const uint64_t al = tc::sdesc(tc::smem_u32(sAl) + oa, lboA, 128);
          const uint64_t bh = tc::sdesc(tc::smem_u32(sBh) + ob, lboB, 128);
          const uint64_t bl = tc::sdesc(tc::smem_u32(sBl) + ob, lboB, 128);
          tc::mma_tf32(tmem, ah, bh, idesc, c > 0 || ks > 0);
          tc::mma_tf32(tmem, ah, bl, idesc, true);
          tc::mma_tf32(tmem, al, bh, idesc, true);
        }
      }
      tc::mma_commit(&empty_bar[st]);   // stage free (and, for the last chunk, D complete)
    }
  }
  // every MMA issued before the last commit has completed once its phase flips
  const int last = nchunk - 1;
  bool ok = tc::mbar_wait(&empty_bar[last & 1], (last >> 1) & 1);
  ok = __syncthreads_and(ok && !abort_flag);
  tc::fence_after();
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
  } else if (warp < 4) {
    // epilogue: lane m of TMEM = row m; every lane of the warp takes part in the loads
    const int m = tid, pl = m >> 6, j = m & 63;
    const bool mine = j < nj;
    const int pi = mine ? j / nbc : 0, b = mine ? j % nbc : 0;
    const int ld = B.db[Th.ix];
    float* out = hsp + ((long long)spt[pi] * 2 + pl) * 4 * nxy + (long long)Th.outq * nxy + Th.ooff +
                 (long long)(Th.b0 + b) * ld + Th.a0;
    for (int n0 = 0; n0 < NP; n0 += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)n0, v);
      if (mine) {
#pragma unroll
        for (int i = 0; i < 8; ++i)
          if (n0 + i < Th.na) out[n0 + i] = 2.f * v[i];
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tmem, ncols);
}

// ---------------------------------------------------------------------------
// Green's function update: vout = G o (q*H + F); layout [P][Re X|Y[|P|Q], Im ...]
// ---------------------------------------------------------------------------
// the Green's function of the points flagged in mask, once per point (omega is fixed):
// G = -1/(E1 + E2 -/+ w) on X (quadrant 0, -w) and Y (1, +w) and, in the statistical
// FAM (nq = 4), G = -1/(E1 - E2 -/+ w) on P (2) and Q (3) (pnfam_solver.f90:420-442),
// times the occupation factor 1 - f1 - f2 (X, Y) or f2 - f1 (P, Q) (:445-458), which
// the reference applies to G o H; gfn: [P][Re | Im][nq*nxy]
__global__ void k_green_prep(long long nxy, int nq, const int* __restrict__ erow, const int* __restrict__ ecol,
                             const double* __restrict__ E1, const double* __restrict__ E2,
                             const double* __restrict__ f1, const double* __restrict__ f2,
                             const double* __restrict__ wre, const double* __restrict__ wim,
                             double* __restrict__ gfn, const int* __restrict__ mask) {
  const int p = blockIdx.y;
  if (!mask[p]) return;
  const long long n2 = nq * nxy;
  const double wr = wre[p], wi = wim[p];
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n2; e += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(e / nxy);
    const double sgn = (q & 1) ? 1.0 : -1.0;
    const double c2 = q < 2 ? 1.0 : -1.0;
    const int r = erow[e], k = ecol[e];
    const double dr = E1[r] + c2 * E2[k] + sgn * wr, di = sgn * wi;
    const double den = dr * dr + di * di;
    double gr = -dr / den, gi = di / den;
    if (f1) {
      const double t = q < 2 ? (-f1[r] - f2[k]) + 1.0 : (-f1[r] + f2[k]) + 0.0;
      gr *= t; gi *= t;
    }
    gfn[(long long)p * 2 * n2 + e] = gr;
    gfn[(long long)p * 2 * n2 + n2 + e] = gi;
  }
}

// vout = G o (q*H + F), G from k_green_prep.  corr[p] != 0 (increment evaluation of the
// mixed form): H is the FP32 field of X - X_anchor (hqp32) and vout = G o (q*H) + radd[p],
// radd = g(X_anchor) evaluated in FP64
__global__ void k_green(long long nxy, int nq, int P, const double* __restrict__ hqp, const float* __restrict__ hqp32,
                        const double* __restrict__ fqp, const double* __restrict__ gfn, double quench,
                        double* __restrict__ vout, const int* __restrict__ active,
                        const int* __restrict__ corr, const double* __restrict__ radd,
                        const int* __restrict__ zeroh) {
  const int p = blockIdx.y;
  if (!active[p]) return;
  const long long n2 = nq * nxy;
  const bool cstep = corr && corr[p];
  const bool useh = hqp && !(zeroh && zeroh[p]);  // zeroh: H = 0 (the field of X = 0)
  const long long o = (long long)p * 2 * n2;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n2; e += (long long)gridDim.x * blockDim.x) {
    double hr = 0.0, hi = 0.0;
    if (useh) {
      if (cstep) { hr = quench * (double)hqp32[o + e]; hi = quench * (double)hqp32[o + n2 + e]; }
      else { hr = quench * hqp[o + e]; hi = quench * hqp[o + n2 + e]; }
    }
    if (!cstep) hr += fqp[e];
    const double gr = gfn[o + e], gi = gfn[o + n2 + e];
    double vr = gr * hr - gi * hi, vi = gr * hi + gi * hr;
    if (cstep) { vr += radd[o + e]; vi += radd[o + n2 + e]; }
    vout[o + e] = vr;
    vout[o + n2 + e] = vi;
  }
}

// ---------------------------------------------------------------------------
// Broyden mixing on device (pnfam_broyden.f90:117-216), one independent
// history per point: itp[p] is the point's own Broyden iteration number and
// modep[p] what the step does (BRO_* below)
// ---------------------------------------------------------------------------
enum { BRO_BROYDEN = 0, BRO_LINEAR = 1, BRO_NOMIX = 2 };
struct BroState {
  int N;            // vector length (2*nq*nxy: Re and Im of the QP quadrants)
  int M;            // history size
  double alpha;
  double* vin;      // [P][N]
  double* vout;     // [P][N]
  double* df;       // [P][M][N]
  double* dv;       // [P][M][N]: u = dv + alpha*df for finished columns, raw vin in column inext
  double* part;     // [P][nchunk][NPART] block partials
  int nchunk;
  const int* itp;   // [P] Broyden iteration of each point
  const int* modep; // [P] BRO_*
};
// block partials, [P][BRO_NPART][nchunk] so that their reduction reads consecutive
// chunks: j = 0: max|vout|, 1: |df_ipos|^2, 2 + k: df_k . df_ipos, 66 + k: df_k . vout
enum { BRO_NPART = 2 + 2 * 64 };
__device__ __forceinline__ long long bro_part(int nchunk, int p, int j) { return ((long long)p * BRO_NPART + j) * nchunk; }
enum { BRO_CHUNK = 1024 };          // elements per CTA of the Broyden kernels (4 per thread)

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
  const int e0 = blockIdx.x * BRO_CHUNK, e1 = min(S.N, e0 + BRO_CHUNK);
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
    S.part[bro_part(S.nchunk, p, 0) + blockIdx.x] = m;
    S.part[bro_part(S.nchunk, p, 1) + blockIdx.x] = s;
  }
}

// normalise column ipos by 1/|df_ipos| (and finish its u column) and form the dots
// dd[k] = df_k . df_ipos and wk[k] = df_k . vout for k < iter_used.
// A CTA covers BRO_CHUNK elements: the normalised df_ipos and vout of its chunk
// are staged in shared memory, then each warp takes whole columns (k = warp,
// warp + 8, ...), every lane streaming its share of the column with many loads
// in flight, and one shuffle reduction per column.
__global__ void __launch_bounds__(256) k_bro_dots(BroState S, const double* __restrict__ norm,
                                                  const int* __restrict__ active) {
  const int p = blockIdx.y;
  if (!active[p]) return;
  const int it = S.itp[p], mode = S.modep[p];
  if (mode != BRO_BROYDEN || it < 1) return;
  int iu, ipos, inext;
  bro_slots(it, S.M, iu, ipos, inext);
  const bool upd = it >= 2;
  __shared__ double sf[BRO_CHUNK], sv[BRO_CHUNK];
  const double* vo = S.vout + (long long)p * S.N;
  double* dfp = S.df + (long long)p * S.M * S.N;
  double* dvp = S.dv + (long long)p * S.M * S.N;
  const long long base = (long long)blockIdx.x * BRO_CHUNK;
  const int len = (int)min((long long)BRO_CHUNK, (long long)S.N - base);
  const double sc = upd ? norm[p] : 0.0;
  for (int i = threadIdx.x; i < BRO_CHUNK; i += blockDim.x) {
    double f = 0.0, v = 0.0;
    if (i < len) {
      const long long e = base + i;
      if (upd) {
        f = dfp[(long long)ipos * S.N + e] * sc;
        dfp[(long long)ipos * S.N + e] = f;
        // the finished dv column is kept as u = dv + alpha*df, the only combination
        // of the two that the update reads
        dvp[(long long)ipos * S.N + e] = fma(S.alpha, f, dvp[(long long)ipos * S.N + e] * sc);
      }
      v = vo[e];
    }
    sf[i] = f;
    sv[i] = v;
  }
  __syncthreads();
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  double* pt = S.part + bro_part(S.nchunk, p, 0) + blockIdx.x;
  for (int k = w; k < iu; k += 8) {
    double a = 0.0, b = 0.0;
    if (k == ipos && upd) {  // column ipos itself: its normalised values are in shared memory
      for (int j = l; j < len; j += 32) {
        const double f = sf[j];
        a = fma(f, f, a);
        b = fma(f, sv[j], b);
      }
    } else {
      const double* fk = dfp + (long long)k * S.N + base;
      if (len == BRO_CHUNK) {  // 16 loads of each lane in flight at a time
        for (int h = 0; h < BRO_CHUNK; h += 16 * 32) {
          double fv[16];
#pragma unroll
          for (int u = 0; u < 16; ++u) fv[u] = __ldcs(fk + h + u * 32 + l);
#pragma unroll
          for (int u = 0; u < 16; ++u) {
            a = fma(fv[u], sf[h + u * 32 + l], a);
            b = fma(fv[u], sv[h + u * 32 + l], b);
          }
        }
      } else {
        for (int j = l; j < len; j += 32) {
          const double f = fk[j];
          a = fma(f, sf[j], a);
          b = fma(f, sv[j], b);
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (l == 0) { pt[(long long)(2 + k) * S.nchunk] = a; pt[(long long)(2 + 64 + k) * S.nchunk] = b; }
  }
}

// one CTA (256 threads) per point: reduce partials; stage 0: si and 1/|df_ipos|;
// stage 1: maintain beta (M x M) and solve beta*gamma = work.  beta is the Gram
// matrix of the unit vectors df_k plus w0^2 on the diagonal, symmetric positive
// definite (the reference factorises it with DSYTRF/DSYTRI, pnfam_broyden.f90:190-206):
// here L D L^T without pivoting, one barrier per column, then two triangular solves
// by one warp
__global__ void __launch_bounds__(256) k_bro_solve(BroState S, int stage, double w0, double* __restrict__ si,
                                                   double* __restrict__ norm, double* __restrict__ beta,
                                                   double* __restrict__ gamma, const int* __restrict__ active) {
  const int p = blockIdx.x;
  if (!active[p]) return;
  const double* pt = S.part + bro_part(S.nchunk, p, 0);
  const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
  __shared__ double red[8][2];
  if (stage == 0) {
    double m = 0.0, s = 0.0;
    for (int c = tid; c < S.nchunk; c += blockDim.x) { m = fmax(m, pt[c]); s += pt[S.nchunk + c]; }
    for (int o = 16; o > 0; o >>= 1) {
      m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
      s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    if (l == 0) { red[w][0] = m; red[w][1] = s; }
    __syncthreads();
    if (tid == 0) {
      double mm = 0.0, ss = 0.0;
      for (int i = 0; i < 8; ++i) { mm = fmax(mm, red[i][0]); ss += red[i][1]; }
      si[p] = mm;
      norm[p] = ss > 0.0 ? 1.0 / sqrt(ss) : 0.0;
    }
    return;
  }
  const int it = S.itp[p], mode = S.modep[p];
  if (mode != BRO_BROYDEN || it < 1) return;
  int n, ipos, inext;
  bro_slots(it, S.M, n, ipos, inext);
  __shared__ double A[64][65];
  __shared__ double x[64];
  __shared__ double dinv[2];   // 1/D of the current and the next column
  const int M = S.M;
  double* bp = beta + (long long)p * M * M;
  for (int k = w; k < n; k += 8) {   // one warp per k: sum the chunk partials
    double dd = 0.0, wk = 0.0;
    const double* pd = pt + (long long)(2 + k) * S.nchunk;
    const double* pw = pt + (long long)(2 + 64 + k) * S.nchunk;
#pragma unroll 4
    for (int c = l; c < S.nchunk; c += 32) { dd += pd[c]; wk += pw[c]; }
    for (int o = 16; o > 0; o >>= 1) {
      dd += __shfl_xor_sync(0xffffffffu, dd, o);
      wk += __shfl_xor_sync(0xffffffffu, wk, o);
    }
    if (l == 0) {
      if (k != ipos) { bp[k * M + ipos] = dd; bp[ipos * M + k] = dd; }
      x[k] = wk;
    }
  }
  __syncthreads();
  for (int k = tid; k < n; k += blockDim.x) bp[k * M + k] = w0 * w0 + 1.0;
  __syncthreads();
  for (int e = tid; e < n * n; e += blockDim.x) A[e / n][e % n] = bp[(e / n) * M + (e % n)];
  if (tid == 0 && n > 0) dinv[0] = 1.0 / A[0][0];
  __syncthreads();
  // L D L^T in place: D on the diagonal, L[r][c] (r > c) in the upper triangle A[c][r]
  for (int c = 0; c < n; ++c) {
    const double di = dinv[c & 1];
    for (int r = c + 1 + w; r < n; r += 8) {
      const double lr = A[r][c] * di;
      for (int j = c + 1 + l; j <= r; j += 32) A[r][j] -= lr * A[j][c];
      if (l == 0) A[c][r] = lr;
      // the next pivot is final as soon as its own update is done (warp 0, lane 0)
      if (r == c + 1 && l == 0) dinv[(c + 1) & 1] = 1.0 / A[r][r];
    }
    __syncthreads();
  }
  // L y = work, y /= D, L^T gamma = y (columns in turn, one warp)
  if (tid < 32) {
    for (int c = 0; c < n; ++c) {
      const double yc = x[c];
      for (int r = c + 1 + tid; r < n; r += 32) x[r] -= A[c][r] * yc;
      __syncwarp();
    }
    for (int r = tid; r < n; r += 32) x[r] /= A[r][r];
    __syncwarp();
    for (int c = n - 1; c >= 0; --c) {
      const double gc = x[c];
      for (int r = tid; r < c; r += 32) x[r] -= A[r][c] * gc;
      __syncwarp();
    }
    for (int k = tid; k < n; k += 32) gamma[(long long)p * 64 + k] = x[k];
  }
}

// BRO_BROYDEN: curv = alpha*vout - sum_i gamma_i u_i  (u_i = dv_i + alpha df_i);
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
    const double* up = S.dv + (long long)p * S.M * S.N;
    for (int k = 0; k < iu; ++k) c -= g[k] * up[(long long)k * S.N + e];
    const double old = vi[e];
    S.df[((long long)p * S.M + inext) * S.N + e] = v;
    S.dv[((long long)p * S.M + inext) * S.N + e] = old;
    vi[e] = old + c;
  }
}

// ---------------------------------------------------------------------------
// Broyden of the mixed form.  The history columns df_k and u_k are kept as pairs
// of floats (hi + lo, about 48 significant bits) and every product with them is
// formed in pair arithmetic on the FP32 cores, which GB300 runs at dozens of times
// its FP64 rate; the raw vout and vin of the previous step and this step's raw
// differences stay FP64, so the secant pairs are formed before any rounding, and
// the small solve is FP64 (k_bro_solve).  Same steps as k_bro_diff / k_bro_dots /
// k_bro_update.
// ---------------------------------------------------------------------------
struct BroState2 {
  int N;              // vector length (4*nxy)
  int M;              // history size
  double alpha;
  double* vin;        // [P][N]
  double* vout;       // [P][N]
  float2* df;         // [P][M][N] finished columns df_k
  float2* u;          // [P][M][N] finished columns u_k = dv_k + alpha*df_k
  double* lastf;      // [P][N] raw vout of the previous step
  double* lastv;      // [P][N] raw vin of the previous step
  double* tf;         // [P][N] vout - lastf of this step (unnormalised)
  double* tv;         // [P][N] vin - lastv of this step
  double* part;       // [P][BRO_NPART][nchunk]
  int nchunk;
  const int* itp;
  const int* modep;
};

__device__ __forceinline__ float2 pair_split(double x) {
  const float h = __double2float_rn(x);
  return make_float2(h, __double2float_rn(x - (double)h));
}
__device__ __forceinline__ double pair_value(float2 a) { return (double)a.x + (double)a.y; }

// s += a*b in pair arithmetic: the exact error of the leading product (FMA) and the
// cross terms go to the low part, the leading sum is a two-sum (rounded operations
// that the compiler may not contract)
__device__ __forceinline__ void pair_fma(float2& s, float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  const float t = __fadd_rn(s.x, p);
  const float z = __fsub_rn(t, s.x);
  const float err = __fadd_rn(__fsub_rn(s.x, __fsub_rn(t, z)), __fsub_rn(p, z));
  s.x = t;
  s.y = __fadd_rn(s.y, __fadd_rn(err, e));
}

// vout -= vin; max|vout|; tf = vout - lastf, tv = vin - lastv, |tf|^2
__global__ void __launch_bounds__(256) k_bro_diff2(BroState2 S, const int* __restrict__ active) {
  const int p = blockIdx.y;
  if (!active[p]) return;
  __shared__ double sh[32];
  const int it = S.itp[p], mode = S.modep[p];
  const bool upd = mode == BRO_BROYDEN && it >= 2;
  const long long o = (long long)p * S.N;
  double mx = 0.0, nn = 0.0;
  const int e0 = blockIdx.x * BRO_CHUNK, e1 = min(S.N, e0 + BRO_CHUNK);
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const double vi = S.vin[o + e];
    const double v = S.vout[o + e] - vi;
    S.vout[o + e] = v;
    mx = fmax(mx, fabs(v));
    if (upd) {
      const double f = v - S.lastf[o + e];
      S.tf[o + e] = f;
      S.tv[o + e] = vi - S.lastv[o + e];
      nn = fma(f, f, nn);
    }
  }
  const double m = block_max(mx, sh);
  const double s = block_sum(nn, sh);
  if (threadIdx.x == 0) {
    S.part[bro_part(S.nchunk, p, 0) + blockIdx.x] = m;
    S.part[bro_part(S.nchunk, p, 1) + blockIdx.x] = s;
  }
}

// finish column ipos (df = tf/|tf|, u = tv/|tf| + alpha*df, stored as pairs) and form
// the dots dd[k] = df_k . df_ipos and wk[k] = df_k . vout, one warp per column
__global__ void __launch_bounds__(256) k_bro_dots2(BroState2 S, const double* __restrict__ norm,
                                                   const int* __restrict__ active) {
  const int p = blockIdx.y;
  if (!active[p]) return;
  const int it = S.itp[p], mode = S.modep[p];
  if (mode != BRO_BROYDEN || it < 1) return;
  int iu, ipos, inext;
  bro_slots(it, S.M, iu, ipos, inext);
  const bool upd = it >= 2;
  __shared__ float2 sf[BRO_CHUNK], sv[BRO_CHUNK];
  const long long o = (long long)p * S.N;
  float2* dfp = S.df + (long long)p * S.M * S.N;
  float2* up = S.u + (long long)p * S.M * S.N;
  const long long base = (long long)blockIdx.x * BRO_CHUNK;
  const int len = (int)min((long long)BRO_CHUNK, (long long)S.N - base);
  const double sc = upd ? norm[p] : 0.0;
  for (int i = threadIdx.x; i < BRO_CHUNK; i += blockDim.x) {
    float2 f2 = make_float2(0.f, 0.f), v2 = f2;
    if (i < len) {
      const long long e = base + i;
      if (upd) {
        const double fn = S.tf[o + e] * sc;
        f2 = pair_split(fn);
        dfp[(long long)ipos * S.N + e] = f2;
        up[(long long)ipos * S.N + e] = pair_split(fma(S.alpha, fn, S.tv[o + e] * sc));
      }
      v2 = pair_split(S.vout[o + e]);
    }
    sf[i] = f2;
    sv[i] = v2;
  }
  __syncthreads();
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  double* pt = S.part + bro_part(S.nchunk, p, 0) + blockIdx.x;
  for (int k = w; k < iu; k += 8) {
    float2 a = make_float2(0.f, 0.f), b = a;
    if (k == ipos && upd) {   // the new column itself: its values are in shared memory
      for (int j = l; j < len; j += 32) {
        pair_fma(a, sf[j], sf[j]);
        pair_fma(b, sf[j], sv[j]);
      }
    } else {
      const float2* fk = dfp + (long long)k * S.N + base;
#pragma unroll 8
      for (int j = l; j < len; j += 32) {
        const float2 x = __ldcs(fk + j);
        pair_fma(a, x, sf[j]);
        pair_fma(b, x, sv[j]);
      }
    }
    double ad = pair_value(a), bd = pair_value(b);
    for (int of = 16; of > 0; of >>= 1) {
      ad += __shfl_xor_sync(0xffffffffu, ad, of);
      bd += __shfl_xor_sync(0xffffffffu, bd, of);
    }
    if (l == 0) { pt[(long long)(2 + k) * S.nchunk] = ad; pt[(long long)(2 + 64 + k) * S.nchunk] = bd; }
  }
}

// BRO_BROYDEN: vin += alpha*vout - sum_k gamma_k u_k; lastf = vout, lastv = vin (raw)
// BRO_LINEAR:  vin += alpha*vout;  BRO_NOMIX: vin += vout
__global__ void __launch_bounds__(256) k_bro_update2(BroState2 S, const double* __restrict__ gamma,
                                                     const int* __restrict__ active) {
  const int p = blockIdx.y;
  if (!active[p]) return;
  const int it = S.itp[p], mode = S.modep[p];
  int iu, ipos, inext;
  bro_slots(it, S.M, iu, ipos, inext);
  if (mode != BRO_BROYDEN) iu = 0;
  const long long o = (long long)p * S.N;
  __shared__ float2 g[64];
  if (mode == BRO_BROYDEN && (int)threadIdx.x < iu) g[threadIdx.x] = pair_split(gamma[(long long)p * 64 + threadIdx.x]);
  __syncthreads();
  const float2* up = S.u + (long long)p * S.M * S.N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < S.N; e += (long long)gridDim.x * blockDim.x) {
    const double v = S.vout[o + e];
    if (mode == BRO_NOMIX) { S.vin[o + e] += v; continue; }
    if (mode == BRO_LINEAR) { S.vin[o + e] += S.alpha * v; continue; }
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll 4
    for (int k = 0; k < iu; ++k) pair_fma(acc, up[(long long)k * S.N + e], g[k]);
    const double old = S.vin[o + e];
    S.lastf[o + e] = v;
    S.lastv[o + e] = old;
    S.vin[o + e] = old + (S.alpha * v - pair_value(acc));
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
// fops: [nops][nq*nxy]; part: [P][nchunk][2*nops]
__global__ void __launch_bounds__(256) k_contract(long long nxy, int nq, int nops, const double* __restrict__ fops,
                                                  const double* __restrict__ vin, int nchunk,
                                                  double* __restrict__ part, const int* __restrict__ active) {
  const int p = blockIdx.y;
  if (!active[p]) return;
  __shared__ double sh[32];
  const long long n2 = nq * nxy;
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
    // one atomic per block: warp maxima, then the block's (a non-negative double orders
    // like its bit pattern)
    __shared__ double wm[32];
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      double b = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b = fmax(b, wm[w]);
      atomicMax(dmax + p, (unsigned long long)__double_as_longlong(b));
    }
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
