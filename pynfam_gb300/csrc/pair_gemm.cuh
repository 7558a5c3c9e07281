// pair_gemm.cuh -- the densities and the field projection of the FP32 increment
// evaluations as GEMMs against a constant pair tensor (tcgen05, 3xTF32, operands
// moved by the bulk-copy engine).
//
// Every density and every field projection of the residual interaction is linear
// in products of two basis functions at one mesh point
// (pnfam_hamiltonian_blas.f90:124-711 densities, :1107-1167 and :1212-1260 the
// projections):
//   density     C_k(q, q', r) = sum_{e in E_k} phi_q(a_e, r) phi_q'(b_e, r) rho_e
//   projection  h_e = 2 sum_{(iy, iz), r} phi_iy(a_e, r) phi_iz(b_e, r) mf(iy, iz, s_a, s_b)(r)
// where e = (a, b) runs over the elements of a block structure whose row state a
// and column state b have the spins of class k = 2 (s_a < 0) + (s_b < 0).  The
// products T_e(c, r) = phi(a_e, r) phi(b_e, r) depend only on the ground state and
// the operator's block structure, so they are formed once per operator (split into
// TF32 hi and lo, laid out in the tensor cores' canonical K-major layout, 128 x 16
// per chunk) and both stages become plain GEMMs of that constant operand against
// the small per-evaluation operand of every active point (rho, or the field
// tensor): D[m][n] = sum_k A[m][k] B[n][k], M = 128 rows per tile, N = the active
// points' columns (Re, Im, both calls), K chunks of 16.  One thread streams the
// chunks of A and B into a ring of shared-memory stages with cp.async.bulk, one
// thread issues the MMAs into a TMEM accumulator, four warps read it out.
//
// Problems (one per block structure, class, stage):
//   projection, mean field   structure F (fc), 18 component pairs, both calls
//   projection, pairing      structures X (xc, call 0) and Y (yc, call 1), (0, 0)
//   density                  structure F, 16 pairs (q, q' < 4), both calls
//   pairing density          structures X^T (xtc, call 0) and Y^T (ytc, call 1), (0, 0)
// A projection problem has rows = elements and K = (pair, mesh point); a density
// problem has rows = (pair, mesh point) and K = elements (split over CTAs, the
// partial sums added by the fold).
#pragma once
#include "tc.cuh"

namespace pnfam {

enum { PG_K = 16, PG_M = 128, PG_MAXN = 256, PG_THREADS = 192, PG_MAXSTAGE = 8, PG_MAXPTS = 64 };
// floats per A chunk (128 rows x 16, hi then lo) and per B chunk slot (up to 256 rows)
constexpr long long PG_ACHUNK = 2LL * PG_M * PG_K;
constexpr long long PG_BCHUNK = 2LL * PG_MAXN * PG_K;

// the (row component, column component) pairs the mean field sets (k_meanfield:
// mf(iy, iz, sa, sb)); the density pairs are all (q, q') with q, q' < 4, c = 4 q + q'
__constant__ signed char c_pg_pairs[18][2] = {{0, 0}, {0, 1}, {1, 0}, {0, 2}, {2, 0}, {0, 3},
                                               {3, 0}, {0, 4}, {4, 0}, {1, 1}, {1, 2}, {2, 1},
                                               {1, 3}, {3, 1}, {2, 2}, {2, 3}, {3, 2}, {3, 3}};
__device__ __forceinline__ void pg_proj_pair(int c, int& iy, int& iz) {
  iy = c_pg_pairs[c][0];
  iz = c_pg_pairs[c][1];
}

struct PGElem {       // one block-matrix element: global row state, column state, offset
  int ja, jb;
  long long off;
};

struct PGProb {
  int kind;           // 0 projection, 1 density
  int pairing;        // 1: pairing field / pairing density (one pair (0, 0))
  int ncombo;         // 18, 16 or 1
  int cls;            // spin class 2 (s_a < 0) + (s_b < 0)
  int ncol;           // columns per point: 4 (Re, Im of both calls) or 2 (one call)
  int call;           // the call of a one-call problem
  long long e0;       // first element in the element table
  int ne;             // elements
  int mrows;          // rows: projection ne, density ncombo * nghl
  int kdim;           // K: projection ncombo * nghl, density ne
  int nkc;            // K chunks
  int ntile;          // M tiles
  int nsplit;         // density: K splits
  long long a0;       // first A chunk (tile t, chunk kc at a0 + t * nkc + kc)
  long long b0;       // first B chunk slot
  long long d0;       // density: float offset of [nsplit][ncol * PG_MAXPTS][mrows] partial sums
};

struct PGTask { int prob, tile, kc0, nkc, split, pad_; };

// ---------------------------------------------------------------------------
// the constant operand, once per operator: grid (A chunks), 256 threads;
// chunks = (problem, tile, chunk) of every A chunk
// ---------------------------------------------------------------------------
struct PGAChunk { int prob, tile, kc, pad_; };

__global__ void __launch_bounds__(256) k_pg_build(const float* __restrict__ phi, int dqp, int nghl,
                                                  const PGProb* __restrict__ probs,
                                                  const PGElem* __restrict__ elems,
                                                  const PGAChunk* __restrict__ chunks, float* __restrict__ apool) {
  const PGAChunk ch = chunks[blockIdx.x];
  const PGProb pr = probs[ch.prob];
  const long long ps = (long long)dqp * nghl;
  float* dst = apool + (pr.a0 + (long long)ch.tile * pr.nkc + ch.kc) * PG_ACHUNK;
  for (int e = threadIdx.x; e < PG_M * PG_K; e += blockDim.x) {
    const int m = e / PG_K, kk = e % PG_K;
    const int row = ch.tile * PG_M + m, k = ch.kc * PG_K + kk;
    float v = 0.f;
    if (row < pr.mrows && k < pr.kdim) {
      int el, c, r;
      if (pr.kind == 0) { el = row; c = k / nghl; r = k % nghl; }   // rows elements, K (pair, r)
      else { el = k; c = row / nghl; r = row % nghl; }              // rows (pair, r), K elements
      int q1 = 0, q2 = 0;
      if (!pr.pairing) {
        if (pr.kind == 0) pg_proj_pair(c, q1, q2);
        else { q1 = c >> 2; q2 = c & 3; }
      }
      const PGElem x = elems[pr.e0 + el];
      v = phi[q1 * ps + (long long)x.ja * nghl + r] * phi[q2 * ps + (long long)x.jb * nghl + r];
    }
    float hi, lo;
    tc::split(v, hi, lo);
    const int o = tc::cm_off(m, kk, PG_M);
    dst[o] = hi;
    dst[PG_M * PG_K + o] = lo;
  }
}

// ---------------------------------------------------------------------------
// per-evaluation operands (B, N = ncol * nact rows padded to 16), split into TF32
// hi and lo: grid (B chunks of the stage), 256 threads; bchunks = (problem, chunk)
// ---------------------------------------------------------------------------
struct PGBChunk { int prob, kc; };

// density: rho (quadrant 0 / 3 of the SP density, or the pairing quadrants 1 / 2)
// of the active points; rsp: [P][2 planes][4 quadrants][nxy]
__global__ void __launch_bounds__(256) k_pg_pack_rho(const PGProb* __restrict__ probs,
                                                     const PGElem* __restrict__ elems,
                                                     const PGBChunk* __restrict__ bchunks,
                                                     const int* __restrict__ actlist, int nact,
                                                     const float* __restrict__ rsp, long long nxy,
                                                     float* __restrict__ bpool) {
  const PGBChunk ch = bchunks[blockIdx.x];
  const PGProb pr = probs[ch.prob];
  const int ncolu = pr.ncol * nact, npad = (ncolu + 15) & ~15;
  float* dst = bpool + (pr.b0 + ch.kc) * PG_BCHUNK;
  for (int e = threadIdx.x; e < npad * PG_K; e += blockDim.x) {
    const int n = e / PG_K, kk = e % PG_K;
    const int el = ch.kc * PG_K + kk;
    float v = 0.f;
    if (n < ncolu && el < pr.ne) {
      const int pi = n / pr.ncol, rem = n % pr.ncol;
      const int call = pr.ncol == 4 ? rem >> 1 : pr.call, plane = pr.ncol == 4 ? (rem & 1) : rem;
      const int quad = pr.pairing ? (call ? 2 : 1) : (call ? 3 : 0);
      const long long p = actlist[pi];
      v = rsp[(p * 2 + plane) * 4 * nxy + (long long)quad * nxy + elems[pr.e0 + el].off];
    }
    float hi, lo;
    tc::split(v, hi, lo);
    const int o = tc::cm_off(n, kk, npad);
    dst[o] = hi;
    dst[npad * PG_K + o] = lo;
  }
}

// projection: the field tensor mf: [P][2 calls][NMF][2 planes][nghl]
__global__ void __launch_bounds__(256) k_pg_pack_field(const PGProb* __restrict__ probs,
                                                       const PGBChunk* __restrict__ bchunks,
                                                       const int* __restrict__ actlist, int nact,
                                                       const float* __restrict__ mf, int nghl,
                                                       float* __restrict__ bpool) {
  const PGBChunk ch = bchunks[blockIdx.x];
  const PGProb pr = probs[ch.prob];
  const int ncolu = pr.ncol * nact, npad = (ncolu + 15) & ~15;
  const int sa = (pr.cls & 2) ? -1 : 1, sb = (pr.cls & 1) ? -1 : 1;
  float* dst = bpool + (pr.b0 + ch.kc) * PG_BCHUNK;
  for (int e = threadIdx.x; e < npad * PG_K; e += blockDim.x) {
    const int n = e / PG_K, kk = e % PG_K;
    const int k = ch.kc * PG_K + kk;
    float v = 0.f;
    if (n < ncolu && k < pr.kdim) {
      const int pi = n / pr.ncol, rem = n % pr.ncol;
      const int call = pr.ncol == 4 ? rem >> 1 : pr.call, plane = pr.ncol == 4 ? (rem & 1) : rem;
      const int c = k / nghl, r = k % nghl;
      int slot;
      if (pr.pairing) {
        slot = 100 + (sa < 0 ? 2 : 0) + (sb < 0 ? 1 : 0);
      } else {
        int iy, iz;
        pg_proj_pair(c, iy, iz);
        slot = mfslot(iy, iz, sa, sb);
      }
      const long long p = actlist[pi];
      v = mf[((p * 2 + call) * NMF + slot) * 2LL * nghl + (long long)plane * nghl + r];
    }
    float hi, lo;
    tc::split(v, hi, lo);
    const int o = tc::cm_off(n, kk, npad);
    dst[o] = hi;
    dst[npad * PG_K + o] = lo;
  }
}

// ---------------------------------------------------------------------------
// the GEMM: one CTA per task (problem, M tile, K range); warp 0 lane 0 streams the
// chunks, warp 1 allocates TMEM and lane 0 issues the MMAs, warps 2-5 read D out.
// bslot: floats of one B stage (>= the widest N of the launch x 64).  Every wait is
// bounded; a CTA whose wait gives up writes nothing and sets *err.
// Projection tasks write hsp [P][2 planes][4 quadrants][nxy] (x 2); density tasks
// write their partial sums dsum + d0 + (split * ncol * PG_MAXPTS + n) * mrows + row.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr size_t pg_smem_bytes(int nstage, int bslot) {
  return (size_t)nstage * ((size_t)PG_ACHUNK + (size_t)bslot) * sizeof(float);
}

__global__ void __launch_bounds__(PG_THREADS, 1) k_pg_gemm(const PGProb* __restrict__ probs,
                                                           const PGTask* __restrict__ tasks,
                                                           const PGElem* __restrict__ elems,
                                                           const float* __restrict__ apool,
                                                           const float* __restrict__ bpool, int nact,
                                                           const int* __restrict__ actlist, int nstage, int bslot,
                                                           float* __restrict__ hsp, long long nxy,
                                                           float* __restrict__ dsum, int* __restrict__ err) {
  const PGTask t = tasks[blockIdx.x];
  const PGProb pr = probs[t.prob];
  const int ncolu = pr.ncol * nact, npad = (ncolu + 15) & ~15;
  extern __shared__ __align__(16) unsigned char smraw[];
  float* sA = reinterpret_cast<float*>(smraw);
  float* sB = sA + (size_t)nstage * PG_ACHUNK;
  __shared__ __align__(8) uint64_t full_bar[PG_MAXSTAGE], empty_bar[PG_MAXSTAGE], done_bar;
  __shared__ uint32_t tslot;
  __shared__ volatile int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ncols = npad <= 32 ? 32u : npad <= 64 ? 64u : npad <= 128 ? 128u : 256u;
  if (threadIdx.x == 0) {
    for (int s = 0; s < nstage; ++s) { tc::mbar_init(&full_bar[s], 1); tc::mbar_init(&empty_bar[s], 1); }
    tc::mbar_init(&done_bar, 1);
    abort_flag = 0;
  }
  if (warp == 1) tc::tmem_alloc(&tslot, ncols);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tslot;
  const long long ach0 = pr.a0 + (long long)t.tile * pr.nkc + t.kc0;
  const long long bch0 = pr.b0 + t.kc0;
  const uint32_t abytes = (uint32_t)(PG_ACHUNK * sizeof(float));
  const uint32_t bbytes = (uint32_t)npad * PG_K * 2 * (uint32_t)sizeof(float);
  if (warp == 0 && lane == 0) {
    // ---------------- producer ----------------
    int issued = 0;
    for (int kc = 0; kc < t.nkc; ++kc) {
      const int st = kc % nstage;
      if (kc >= nstage && !abort_flag && !tc::mbar_wait(&empty_bar[st], ((kc / nstage) - 1) & 1)) abort_flag = 1;
      if (abort_flag) break;
      tc::mbar_expect_tx(&full_bar[st], abytes + bbytes);
      tc::bulk_g2s(sA + (size_t)st * PG_ACHUNK, apool + (ach0 + kc) * PG_ACHUNK, abytes, &full_bar[st]);
      tc::bulk_g2s(sB + (size_t)st * bslot, bpool + (bch0 + kc) * PG_BCHUNK, bbytes, &full_bar[st]);
      issued = kc + 1;
    }
    // no copy may still be landing when the CTA exits: the last chunk of each stage
    for (int kc = issued > nstage ? issued - nstage : 0; kc < issued; ++kc)
      if (!tc::mbar_wait(&full_bar[kc % nstage], (kc / nstage) & 1)) abort_flag = 1;
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer ----------------
    const uint32_t idesc = tc::idesc_tf32(PG_M, npad);
    const uint32_t lboA = (PG_M / 8) * 128, lboB = (uint32_t)(npad / 8) * 128;
    for (int kc = 0; kc < t.nkc; ++kc) {
      const int st = kc % nstage;
      if (!abort_flag && !tc::mbar_wait(&full_bar[st], (kc / nstage) & 1)) abort_flag = 1;
      if (abort_flag) break;
      tc::fence_after();
      const float* Ah = sA + (size_t)st * PG_ACHUNK;
      const float* Al = Ah + PG_M * PG_K;
      const float* Bh = sB + (size_t)st * bslot;
      const float* Bl = Bh + npad * PG_K;
#pragma unroll
      for (int ks = 0; ks < PG_K / 8; ++ks) {
        const uint32_t oa = ks * 2 * lboA, ob = ks * 2 * lboB;
        const uint64_t ah = tc::sdesc(tc::smem_u32(Ah) + oa, lboA, 128);
        const uint64_t al = tc::sdesc(tc::smem_u32(Al) + oa, lboA, 128);
        const uint64_t bh = tc::sdesc(tc::smem_u32(Bh) + ob, lboB, 128);
        const uint64_t bl = tc::sdesc(tc::smem_u32(Bl) + ob, lboB, 128);
        tc::mma_tf32(tmem, ah, bh, idesc, kc > 0 || ks > 0);
        tc::mma_tf32(tmem, ah, bl, idesc, true);
        tc::mma_tf32(tmem, al, bh, idesc, true);
      }
      tc::mma_commit(&empty_bar[st]);
    }
    tc::mma_commit(&done_bar);   // arrives when every MMA issued above has completed
  }
  bool ok = true;
  if (warp >= 2) ok = tc::mbar_wait(&done_bar, 0);
  ok = __syncthreads_and(ok && !abort_flag && t.nkc > 0);
  tc::fence_after();
  if (!ok) {
    if (threadIdx.x == 0 && t.nkc > 0) atomicExch(err, 1);
  } else if (warp >= 2) {
    const int q = warp & 3;              // TMEM lanes 32q..32q+31 (warp w reaches lanes 32 (w % 4))
    const int m = 32 * q + lane;
    const int row = t.tile * PG_M + m;
    const bool mine = row < pr.mrows;
    const uint32_t tbase = tmem + ((uint32_t)(32 * q) << 16);
    if (pr.kind == 0) {
      const long long off = mine ? elems[pr.e0 + row].off : 0;
      for (int n0 = 0; n0 < npad; n0 += 8) {
        float v[8];
        tc::tmem_ld8(tbase + (uint32_t)n0, v);
        if (mine) {
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const int n = n0 + i;
            if (n >= ncolu) break;
            const int pi = n / pr.ncol, rem = n % pr.ncol;
            const int call = pr.ncol == 4 ? rem >> 1 : pr.call, plane = pr.ncol == 4 ? (rem & 1) : rem;
            const int quad = pr.pairing ? (call ? 2 : 1) : (call ? 3 : 0);
            const long long p = actlist[pi];
            hsp[(p * 2 + plane) * 4 * nxy + (long long)quad * nxy + off] = 2.f * v[i];
          }
        }
      }
    } else {
      float* out = dsum + pr.d0 + (long long)t.split * pr.ncol * PG_MAXPTS * pr.mrows + row;
      for (int n0 = 0; n0 < npad; n0 += 8) {
        float v[8];
        tc::tmem_ld8(tbase + (uint32_t)n0, v);
        if (mine) {
#pragma unroll
          for (int i = 0; i < 8; ++i)
            if (n0 + i < ncolu) out[(long long)(n0 + i) * pr.mrows] = v[i];
        }
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 1) tc::tmem_free(tmem, ncols);
}

// ---------------------------------------------------------------------------
// fold: the class sums C_k(q, q', r) of the density problems into the 28 complex
// densities of each point and call, in the layout k_meanfield reads with G = 1:
// dpart [P][2 calls][2 ND][nghl].  dens: the problem index of the density problem of
// structure F and class k (dens[k]) and of the pairing-density problems of call 0
// (dens[4 + k]) and call 1 (dens[8 + k]).  grid (ceil(nghl / 128), nact, 2 calls)
// ---------------------------------------------------------------------------
struct PGFold { int dens[12]; };

__device__ __forceinline__ void accC(float (&acc)[2 * ND], int k, float re, float im) {
  acc[2 * k] += re;
  acc[2 * k + 1] += im;
}

// same-spin class (row spin = column spin = sg): the terms of dens_same with the row
// sums W_q(r, b) times phi_q'(b, r) summed over the columns, i.e. C(q, q')
__device__ __forceinline__ void fold_same(float (&acc)[2 * ND], const float (&Cr)[16], const float (&Ci)[16],
                                          float sg) {
  const float h5 = 0.5f;
#define CR(i, j) Cr[(i) * 4 + (j)]
#define CI(i, j) Ci[(i) * 4 + (j)]
  float xr, xi;
  xr = CR(0, 0); xi = CI(0, 0);
  accC(acc, D_RHO, xr, xi);
  accC(acc, D_SZ, sg * xr, sg * xi);
  xr = h5 * (CR(0, 2) + CR(2, 0)); xi = h5 * (CI(0, 2) + CI(2, 0));
  accC(acc, D_JP, xr, xi);
  accC(acc, D_TJPZ, sg * xr, sg * xi);
  xr = CR(1, 1) + CR(2, 2) + CR(3, 3); xi = CI(1, 1) + CI(2, 2) + CI(3, 3);
  accC(acc, D_TAU, xr, xi);
  accC(acc, D_TZ, sg * xr, sg * xi);
  xr = h5 * (CR(0, 1) - CR(1, 0)); xi = h5 * (CI(0, 1) - CI(1, 0));
  accC(acc, D_JR, -xi, xr);
  accC(acc, D_TJRZ, -sg * xi, sg * xr);
  xr = h5 * (CR(0, 3) - CR(3, 0)); xi = h5 * (CI(0, 3) - CI(3, 0));
  accC(acc, D_JZ, -xi, xr);
  accC(acc, D_TJZZ, -sg * xi, sg * xr);
  accC(acc, D_GS, sg * (CR(0, 3) + CR(3, 0)), sg * (CI(0, 3) + CI(3, 0)));
  accC(acc, D_FR, h5 * sg * (CR(1, 3) + CR(3, 1)), h5 * sg * (CI(1, 3) + CI(3, 1)));
  {
    const float ar = h5 * sg * (CR(2, 3) - CR(3, 2)), ai = h5 * sg * (CI(2, 3) - CI(3, 2));
    accC(acc, D_FP, -ai, ar);
  }
  accC(acc, D_FZ, sg * CR(3, 3), sg * CI(3, 3));
}

// opposite-spin class: the terms of dens_opp (sig = +1 when the column is spin down)
__device__ __forceinline__ void fold_opp(float (&acc)[2 * ND], const float (&Cr)[16], const float (&Ci)[16],
                                         float sig) {
  const float h5 = 0.5f;
  float xr, xi;
  accC(acc, D_GS, sig * (CR(0, 2) - CR(2, 0)) + (CR(0, 1) + CR(1, 0)),
       sig * (CI(0, 2) - CI(2, 0)) + (CI(0, 1) + CI(1, 0)));
  accC(acc, D_FR, CR(1, 1) + sig * h5 * (CR(1, 2) - CR(2, 1)), CI(1, 1) + sig * h5 * (CI(1, 2) - CI(2, 1)));
  {
    const float ar = sig * CR(2, 2) + h5 * (CR(2, 1) - CR(1, 2));
    const float ai = sig * CI(2, 2) + h5 * (CI(2, 1) - CI(1, 2));
    accC(acc, D_FP, -ai, ar);
  }
  accC(acc, D_FZ, h5 * (CR(3, 1) + sig * CR(3, 2) + CR(1, 3) - sig * CR(2, 3)),
       h5 * (CI(3, 1) + sig * CI(3, 2) + CI(1, 3) - sig * CI(2, 3)));
  xr = CR(0, 0); xi = CI(0, 0);
  accC(acc, D_SR, xr, xi);
  accC(acc, D_SP, -sig * xi, sig * xr);
  xr = h5 * (CR(2, 0) + CR(0, 2)); xi = h5 * (CI(2, 0) + CI(0, 2));
  accC(acc, D_TJPR, xr, xi);
  accC(acc, D_TJPP, -sig * xi, sig * xr);
  xr = CR(1, 1) + CR(2, 2) + CR(3, 3); xi = CI(1, 1) + CI(2, 2) + CI(3, 3);
  accC(acc, D_TR, xr, xi);
  accC(acc, D_TP, -sig * xi, sig * xr);
  xr = h5 * (CR(0, 1) - CR(1, 0)); xi = h5 * (CI(0, 1) - CI(1, 0));
  accC(acc, D_TJRR, -xi, xr);
  accC(acc, D_TJRP, -sig * xr, -sig * xi);
  xr = h5 * (CR(0, 3) - CR(3, 0)); xi = h5 * (CI(0, 3) - CI(3, 0));
  accC(acc, D_TJZR, -xi, xr);
  accC(acc, D_TJZP, -sig * xr, -sig * xi);
#undef CR
#undef CI
}

// sum of the K splits of one column n of a density problem at row `row`
__device__ __forceinline__ float pg_dsum(const float* __restrict__ dsum, const PGProb& pr, int n, int row) {
  float s = 0.f;
  const long long stride = (long long)pr.ncol * PG_MAXPTS * pr.mrows;
  const float* p = dsum + pr.d0 + (long long)n * pr.mrows + row;
  for (int sp = 0; sp < pr.nsplit; ++sp) s += p[sp * stride];
  return s;
}

// one thread per (mesh point, class): the class's terms go into shared memory and are
// added over the four classes in a fixed order.  grid (ceil(nghl / PG_FOLD_R), nact,
// 2 calls), block 4 * PG_FOLD_R
enum { PG_FOLD_R = 32 };

__global__ void __launch_bounds__(4 * PG_FOLD_R) k_pg_fold(const PGProb* __restrict__ probs, PGFold F,
                                                           const float* __restrict__ dsum,
                                                           const int* __restrict__ actlist, int nghl,
                                                           float* __restrict__ dpart) {
  __shared__ float sacc[4][2 * ND][PG_FOLD_R];
  const int rl = threadIdx.x % PG_FOLD_R, cls = threadIdx.x / PG_FOLD_R;
  const int r = blockIdx.x * PG_FOLD_R + rl;
  const int pi = blockIdx.y, call = blockIdx.z;
  float acc[2 * ND];
#pragma unroll
  for (int k = 0; k < 2 * ND; ++k) acc[k] = 0.f;
  const bool rok = r < nghl;
  const float sb = (cls & 1) ? -1.f : 1.f;
  const bool same = ((cls >> 1) & 1) == (cls & 1);
  if (rok && F.dens[cls] >= 0) {
    const PGProb pr = probs[F.dens[cls]];
    float Cr[16], Ci[16];
    const int nre = pi * 4 + call * 2;
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      Cr[c] = pg_dsum(dsum, pr, nre, c * nghl + r);
      Ci[c] = pg_dsum(dsum, pr, nre + 1, c * nghl + r);
    }
    if (same) fold_same(acc, Cr, Ci, sb);
    else fold_opp(acc, Cr, Ci, sb < 0.f ? 1.f : -1.f);
  }
  const int pp = F.dens[4 + 4 * call + cls];
  if (rok && pp >= 0) {
    // pairing densities (the kind-1 terms of the density kernels)
    const PGProb pr = probs[pp];
    const float xr = 2.f * pg_dsum(dsum, pr, pi * 2, r), xi = 2.f * pg_dsum(dsum, pr, pi * 2 + 1, r);
    if (same) {
      const float sig = sb < 0.f ? 1.f : -1.f;
      accC(acc, D_SBR, sig * xr, sig * xi);
      accC(acc, D_SBP, xi, -xr);
    } else {
      accC(acc, D_RB, -sb * xr, -sb * xi);
      accC(acc, D_SBZ, xr, xi);
    }
  }
#pragma unroll
  for (int k = 0; k < 2 * ND; ++k) sacc[cls][k][rl] = acc[k];
  __syncthreads();
  const long long p = actlist[pi];
  float* out = dpart + (p * 2 + call) * (2LL * ND) * nghl;
  for (int e = threadIdx.x; e < 2 * ND * PG_FOLD_R; e += blockDim.x) {
    const int k = e / PG_FOLD_R, q = e % PG_FOLD_R, rr = blockIdx.x * PG_FOLD_R + q;
    if (rr < nghl) out[(long long)k * nghl + rr] = (sacc[0][k][q] + sacc[1][k][q]) + (sacc[2][k][q] + sacc[3][k][q]);
  }
}

}  // namespace pnfam
