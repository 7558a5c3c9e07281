// pnfam_gpu.cu -- C ABI + host orchestration of the GB300 pnFAM solver.
//
// The ground state (U, V, E, basis functions on the mesh, couplings) is
// uploaded once per nucleus; an operator is set once per (O, K, beta); a
// batch of omega points is then iterated in lock step, each point keeping
// its own Broyden history and stopping at its own convergence, exactly as
// the reference's per-process ifam loop (pnfam_solver.f90:114-209) does.
#include "../../include/pnfam_gpu.h"
#include "pnfam_kernels.cuh"
#include "pair_gemm.cuh"
#include "tbc.cuh"
#include "hfb.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <tuple>
#include <type_traits>
#include <mutex>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace pnfam;

static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CK(call)                                                                             \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      return fail(e_ == cudaErrorMemoryAllocation ? PNFAM_ENOMEM : PNFAM_ECUDA,              \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                       \
    }                                                                                        \
  } while (0)

namespace {

// asynchronous FP64 anchor batches an engine keeps in flight at most
constexpr int ANCH_RING = 8;

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

template <class T>
static cudaError_t dalloc(DBuf<T>& b, size_t n) {
  if (b.n >= n && b.p) return cudaSuccess;
  b.release();
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(&b.p, n * sizeof(T));
  if (e == cudaSuccess) b.n = n;
  return e;
}

template <class T>
static cudaError_t upload(DBuf<T>& b, const T* h, size_t n) {
  cudaError_t e = dalloc(b, n);
  if (e != cudaSuccess) return e;
  return cudaMemcpy(b.p, h, n * sizeof(T), cudaMemcpyHostToDevice);
}

struct MatRef {      // op(stored block)
  int buf;
  long long off;
  int rows, cols;    // stored shape
  int trans;
  int orows() const { return trans ? cols : rows; }
  int ocols() const { return trans ? rows : cols; }
};

struct Term2 {       // s * A * T
  double alpha[2];
  MatRef A, T;
};

struct TaskList {
  std::vector<GemmTask> tasks;
  std::vector<int> tile2task;
  DBuf<GemmTask> d_tasks;
  DBuf<int> d_tile2task;
  int ntiles = 0;

  void add(int M, int N, int K, const std::vector<GemmTerm>& terms, int cbuf, long long coff, int ldc) {
    if (M <= 0 || N <= 0) return;
    GemmTask t;
    memset(&t, 0, sizeof(t));
    t.M = M; t.N = N; t.K = K; t.nterm = (int)terms.size();
    for (size_t i = 0; i < terms.size(); ++i) t.t[i] = terms[i];
    t.cbuf = cbuf; t.coff = coff; t.ldc = ldc;
    // tile shape: the fewest 1024-element tiles covering M x N (32 x 32 on ties); every
    // tile costs the same DFMAs, so this is the fewest padded outputs
    int best = 32, bt = -1;
    for (int tm : {32, 64, 16, 128, 8}) {
      const int tn = 1024 / tm;
      const int nt = ((M + tm - 1) / tm) * ((N + tn - 1) / tn);
      if (bt < 0 || nt < bt) { bt = nt; best = tm; }
    }
    t.tm = best;
    const int ntm = (M + best - 1) / best, ntn = (N + 1024 / best - 1) / (1024 / best);
    t.tile0 = ntiles; t.ntn = ntn;
    for (int k = 0; k < ntm * ntn; ++k) tile2task.push_back((int)tasks.size());
    ntiles += ntm * ntn;
    tasks.push_back(t);
  }
  cudaError_t finalize() {
    cudaError_t e = upload(d_tasks, tasks.data(), tasks.size());
    if (e != cudaSuccess) return e;
    return upload(d_tile2task, tile2task.data(), tile2task.size());
  }
  void clear() {
    tasks.clear(); tile2task.clear(); ntiles = 0;
  }
};

// the same tasks for the tensor-core kernel (FP32 data)
struct TaskListTC {
  std::vector<GemmTaskTC> tasks;
  DBuf<GemmTaskTC> d_tasks;
  int maxrows = 0, maxnp = 16;
  void build(const TaskList& tl) {
    tasks.clear();
    maxrows = 0;
    maxnp = 16;
    for (const GemmTask& g : tl.tasks) {
      GemmTaskTC t;
      memset(&t, 0, sizeof(t));
      t.M = g.M; t.N = g.N; t.K = g.K; t.nterm = g.nterm;
      for (int i = 0; i < g.nterm; ++i) t.t[i] = g.t[i];
      t.rcase = g.t[0].abuf >= B_STATE ? 0 : 1;
      t.mrows = t.rcase == 0 ? g.M : g.N;
      t.ncols = t.rcase == 0 ? g.N : g.M;
      t.npad = std::max(16, (t.ncols + 15) / 16 * 16);
      t.coff = g.coff; t.cbuf = g.cbuf; t.ldc = g.ldc;
      maxrows = std::max(maxrows, t.mrows);
      maxnp = std::max(maxnp, t.npad);
      tasks.push_back(t);
    }
  }
};

static GemmTerm mkterm(const MatRef& A, const MatRef& B, double a_re, double a_im) {
  GemmTerm g;
  memset(&g, 0, sizeof(g));
  g.abuf = A.buf; g.aoff = A.off; g.lda = A.rows; g.tA = A.trans;
  g.bbuf = B.buf; g.boff = B.off; g.ldb = B.rows; g.tB = B.trans;
  g.alpha[0] = a_re; g.alpha[1] = a_im;
  return g;
}

}  // namespace

// pinned host memory: a copy between the device and pageable host memory makes the
// host wait (device to pageable host returns only when the stream has reached it),
// which would keep the engines of different contexts from overlapping on the GPU
template <class T>
struct PinBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t m) {
    if (p && n >= m) return cudaSuccess;
    release();
    const cudaError_t e = cudaMallocHost(reinterpret_cast<void**>(&p), std::max<size_t>(m, 1) * sizeof(T));
    if (e == cudaSuccess) n = m; else p = nullptr;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
  }
  ~PinBuf() { release(); }
};

struct pnfam_engine;
struct pnfam_ctx {
  int dev = 0;
  // basis (host)
  int nb = 0, dqp = 0, nghl = 0;
  std::vector<int> db, st, nup, tr;
  std::vector<long long> uoff;
  std::vector<signed char> ns;
  // device ground state
  DBuf<int> d_db, d_st, d_nup;
  DBuf<signed char> d_ns;
  DBuf<double> d_up, d_vp, d_un, d_vn, d_ep, d_en, d_phi, d_wd, d_crho, d_cs, d_cpair, d_cspair;
  double sc[12] = {0};
  // operator
  bool have_op = false;
  int beta_minus = 1;
  long long nxy = 0;
  int nops = 1;
  std::vector<int> fc, xc, yc, xtc, ytc;
  std::vector<long long> foff, xoff, yoff, xtoff, ytoff;
  // statistical FAM (finite temperature, EFA blocking): the diagonal quadrants P
  // (m11) and Q (m22) join X and Y; nq = quadrants of the QP state
  int nq = 2;
  std::vector<int> pc, qc;
  std::vector<long long> poff, qoff;
  DBuf<double> d_fp, d_fn;   // [dqp] quasiparticle occupations
  long long tplane = 0;      // elements per plane of the GEMM scratch (B_T)
  DBuf<int> d_fc, d_xtc, d_ytc, d_erow, d_ecol;
  DBuf<long long> d_foff, d_xtoff, d_ytoff;
  DBuf<double> d_fops;   // [nops][2*nxy] operator and cross terms in the QP basis
  TaskList k1a, k1b, k2a, k2b;
  TaskListTC t1a, t1b, t2a, t2b;   // FP32 evaluation on the tensor cores
  std::vector<HTask> htasks;
  DBuf<HTask> d_htasks;
  DBuf<float> d_gsplit;               // ground-state operands of the tensor-core GEMM tasks, pre-split
  long long gsplit_floats = 0;
  bool have_gsplit = false;
  std::vector<HTaskTC> htasks_tc;   // tensor-core field projection (FP32 data)
  int tc_npmax = 16;                  // largest N of those tiles
  DBuf<HTaskTC> d_htasks_tc;
  std::vector<HPTile> hptiles;        // their row tiles, with the pre-split basis functions
  DBuf<HPTile> d_hptiles;
  DBuf<float> d_hphi;
  long long hphi_floats = 0;
  bool have_hphi = false;
  DBuf<int> d_actlist;   // [P] points of the current FP32 evaluation (tensor-core tiles)
  DBuf<int> d_err;       // set by a tensor-core kernel whose wait gave up
  // per-solve buffers
  int cap_P = 0, cap_M = 0;
  DBuf<double> d_state, d_vout, d_T, d_rsp, d_hsp, d_hqp, d_dpart, d_mf;
  DBuf<double> d_df, d_dv, d_bpart, d_si, d_norm, d_beta, d_gamma, d_cpart, d_wre, d_wim;
  DBuf<double> d_gfn;   // [P][Re | Im][nq*nxy] Green's function of each slot's omega
  DBuf<int> d_active, d_act32, d_act64;
  DBuf<int> d_act64r;   // [ANCH_RING][P] slot flags of the asynchronous anchor batches
  DBuf<int> d_pint;      // [6][P]: Broyden iteration, Broyden mode, increment step, anchor step,
                         // zero field (first evaluation), newly admitted
  DBuf<BufDesc> d_bufs;
  // mixed precision: FP32 copies of the ground state and FP32 scratch
  bool have32 = false;
  DBuf<float> d_up32, d_vp32, d_un32, d_vn32, d_phi32;
  DBuf<float> d_state32, d_T32, d_rsp32, d_hsp32, d_hqp32, d_dpart32, d_mf32;
  DBuf<BufDescT<float>> d_bufs32;
  DBuf<double> d_xsave, d_radd;   // [P][4nxy] mixed form: anchor X_a and its FP64 image g(X_a)
  DBuf<unsigned long long> d_dmax;  // [P] max|X - X_a| of the last increment evaluation
  DBuf<double> d_lastf, d_lastv, d_tf, d_tv;  // [P][4nxy] mixed-form Broyden: raw vectors of the last step, raw differences
  // tensor-core densities: unit tables per call, B chunks to lay out, pre-split A
  std::vector<DUnitTC> dunits[2];
  std::vector<DBChunkTC> bchunks;
  std::vector<DAChunkTC> achunks;
  DBuf<DUnitTC> d_dunits0, d_dunits1;
  DBuf<DBChunkTC> d_bchunks;
  DBuf<DAChunkTC> d_achunks;
  DBuf<float> d_aphi;     // [ceil(nghl/32)][nachunk][DTC2_ACH], once per ground state
  DBuf<float> d_bsplit;   // [P][bstride]
  long long bstride = 0;
  bool have_aphi = false;
  long long pit64 = 0, pit32 = 0;   // point-iterations per precision in the last solve
  int G = 1;
  int nsm = 1;
  int maxdb = 0;
  // FP32 densities on the tensor cores (k_density_tc2, the default) or on the SIMT
  // cores (k_density<float>, PNFAM_GB300_TC_DENSITY=0 at context creation)
  bool tc_density = true;
  // FP32 densities and field projection as GEMMs against the operator's pair tensor
  // (pair_gemm.cuh): PNFAM_GB300_PAIR_GEMM=0 at context creation keeps the kernels
  // above; the pair tensor is formed only while it fits PNFAM_GB300_PAIR_GEMM_GB
  // (default 16 GB), and used for evaluations of at least pg_min points
  int pg_mode = 1;
  double pg_budget = 16e9;
  int pg_min = 4;
  bool pg_on = false, pg_built = false;
  // autotuning (pg_autotune, once per operator, unless PNFAM_GB300_AUTOTUNE=0): the K
  // chunks per density task (pg_kspan) and, unless PNFAM_GB300_PAIR_MIN fixes it,
  // pg_min, the point count from which the pair-tensor path is the faster one
  int pg_kspan = 384;
  int pg_kspan_env = 0;   // PNFAM_GB300_PAIR_KSPAN: a fixed span (no span trials)
  // shared memory of a pair-GEMM CTA (its ring of stages): 104 KB puts two CTAs on an SM,
  // so that one streams the pair tensor while the other starts or drains a task (measured:
  // 73.4 points/s on the benchmark against 72.6 with one 128 KB CTA and 69.5 with 208 KB);
  // PNFAM_GB300_PAIR_SMEM_KB (<= 224) changes it
  int pg_smem = 104 * 1024;
  bool pg_tuned = false, pg_min_env = false, autotune = true;
  double tune_ms = 0.0;
  std::vector<PGProb> pg_probs;
  std::vector<PGElem> pg_elems;
  std::vector<PGTask> pg_tproj, pg_tdens;
  std::vector<PGBChunk> pg_bproj, pg_bdens;
  std::vector<PGAChunk> pg_ach;
  PGFold pg_fold{};
  long long pg_nachunk = 0, pg_nbchunk = 0, pg_dfloats = 0;
  DBuf<PGProb> d_pg_probs;
  DBuf<PGElem> d_pg_elems;
  DBuf<PGTask> d_pg_tproj, d_pg_tdens;
  DBuf<PGBChunk> d_pg_bproj, d_pg_bdens;
  DBuf<float> d_pg_a, d_pg_b, d_pg_d;
  int nchunk_bro = 1, nchunk_c = 1;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaEvent_t evt[2] = {nullptr, nullptr};   // whole-solve device time
  cudaStream_t stream64 = nullptr;           // FP64 anchor evaluations beside the FP32 increments
  cudaEvent_t evf[2] = {nullptr, nullptr};   // fork to / join from stream64
  cudaEvent_t evd = nullptr;                 // end of the engine's evaluation in flight
  double stage_ms[8] = {0};     // FP64 evaluations (0-4) and the common stages (5-7)
  double stage32_ms[5] = {0};   // FP32 evaluations of the mixed form
  // live timing of the FP32 density and field-projection launches (opts.reserved[2]):
  // an event pair around each launch on its own stream, read once the engine has
  // waited for the evaluation, so nothing is serialised or synchronised for it
  bool live = false;
  std::vector<cudaEvent_t> lev;   // [2 * pairs]
  std::vector<int> lkind;         // stage of each pair: 0 density, 1 field projection
  int nlev = 0;
  double live_ms[2] = {0.0, 0.0};
  long long live_n[2] = {0, 0};
  double total_ms = 0.0;
  long long launches = 0;
  pnfam_engine* engine = nullptr;   // the engine using this context's solve buffers
  void detach_engine();

  ~pnfam_ctx() {
    detach_engine();
    DBuf<int>* ib[] = {&d_db, &d_st, &d_nup, &d_fc, &d_xtc, &d_ytc, &d_erow, &d_ecol, &d_active, &d_act32, &d_act64, &d_act64r,
                      &d_pint};
    DBuf<float>* fb[] = {&d_up32, &d_vp32, &d_un32, &d_vn32, &d_phi32, &d_state32, &d_T32, &d_rsp32, &d_hsp32,
                         &d_hqp32, &d_dpart32, &d_mf32};
    for (auto* b : fb) b->release();
    d_bufs32.release();
    d_xsave.release(); d_radd.release(); d_dmax.release();
    d_lastf.release(); d_lastv.release(); d_tf.release(); d_tv.release();
    d_dunits0.release(); d_dunits1.release(); d_bchunks.release(); d_achunks.release(); d_aphi.release();
    d_bsplit.release();
    for (auto* b : ib) b->release();
    d_ns.release();
    DBuf<double>* dbs[] = {&d_up, &d_vp, &d_un, &d_vn, &d_ep, &d_en, &d_phi, &d_wd, &d_crho, &d_cs,
                           &d_cpair, &d_cspair, &d_fops, &d_state, &d_vout, &d_T, &d_rsp, &d_hsp,
                           &d_hqp, &d_dpart, &d_mf, &d_df, &d_dv, &d_bpart, &d_si, &d_norm,
                           &d_beta, &d_gamma, &d_cpart, &d_wre, &d_wim, &d_gfn, &d_fp, &d_fn};
    for (auto* b : dbs) b->release();
    d_foff.release(); d_xtoff.release(); d_ytoff.release();
    d_htasks.release(); d_bufs.release(); d_htasks_tc.release(); d_actlist.release(); d_err.release();
    d_gsplit.release(); d_hptiles.release(); d_hphi.release();
    d_pg_probs.release(); d_pg_elems.release(); d_pg_tproj.release(); d_pg_tdens.release();
    d_pg_bproj.release(); d_pg_bdens.release(); d_pg_a.release(); d_pg_b.release(); d_pg_d.release();
    k1a.d_tasks.release(); k1a.d_tile2task.release();
    k1b.d_tasks.release(); k1b.d_tile2task.release();
    k2a.d_tasks.release(); k2a.d_tile2task.release();
    k2b.d_tasks.release(); k2b.d_tile2task.release();
    t1a.d_tasks.release(); t1b.d_tasks.release(); t2a.d_tasks.release(); t2b.d_tasks.release();
    if (ev[0]) cudaEventDestroy(ev[0]);
    if (ev[1]) cudaEventDestroy(ev[1]);
    if (evt[0]) cudaEventDestroy(evt[0]);
    if (evt[1]) cudaEventDestroy(evt[1]);
    if (evf[0]) cudaEventDestroy(evf[0]);
    if (evf[1]) cudaEventDestroy(evf[1]);
    if (evd) cudaEventDestroy(evd);
    for (cudaEvent_t e : lev) cudaEventDestroy(e);
    if (stream64) cudaStreamDestroy(stream64);
    if (stream) cudaStreamDestroy(stream);
  }

  template <class T>
  DevBasisT<T> devbasis() const {
    DevBasisT<T> B;
    B.nb = nb; B.dqp = dqp; B.nghl = nghl;
    B.db = d_db.p; B.st = d_st.p; B.nup = d_nup.p; B.ns = d_ns.p;
    B.phi = phi_ptr<T>(); B.wdcori = d_wd.p;
    B.crho = d_crho.p; B.cs = d_cs.p; B.cpair = d_cpair.p; B.cspair = d_cspair.p;
    for (int i = 0; i < 12; ++i) B.sc[i] = sc[i];
    return B;
  }
  template <class T> const T* phi_ptr() const;
  int left_u() const { return beta_minus ? B_UP : B_UN; }
  int left_v() const { return beta_minus ? B_VP : B_VN; }
  int right_u() const { return beta_minus ? B_UN : B_UP; }
  int right_v() const { return beta_minus ? B_VN : B_VP; }
  MatRef ublk(int buf, int i, int trans) const { return MatRef{buf, uoff[i], db[i], db[i], trans}; }
  MatRef vblk(int buf, int i, int trans) const { return MatRef{buf, uoff[i], db[i], db[tr[i]], trans}; }
};

template <> const double* pnfam_ctx::phi_ptr<double>() const { return d_phi.p; }
template <> const float* pnfam_ctx::phi_ptr<float>() const { return d_phi32.p; }

// ---------------------------------------------------------------------------
// structures and task lists
// ---------------------------------------------------------------------------
static std::vector<long long> offsets(const std::vector<int>& cols, const std::vector<int>& db, long long* total) {
  std::vector<long long> off(cols.size(), -1);
  long long p = 0;
  for (size_t i = 0; i < cols.size(); ++i)
    if (cols[i] >= 0) { off[i] = p; p += (long long)db[i] * db[cols[i]]; }
  *total = p;
  return off;
}

// Stage-1/stage-2 split of sum_t s_t A_t (op(B_t) C_t'):
// T_t = op(B_t) op(C_t) in scratch, then out = sum_t s_t op(A_t) T_t.
struct TripleTerm {
  double alpha[2];
  MatRef A, B, C;
};

static void emit_triple(TaskList& s1, TaskList& s2, long long& toff, const std::vector<TripleTerm>& terms,
                        int obuf, long long ooff, int orows, int ocols) {
  std::vector<GemmTerm> st2;
  for (const TripleTerm& t : terms) {
    const int M = t.B.orows(), N = t.C.ocols(), K = t.B.ocols();
    MatRef T{B_T, toff, M, N, 0};
    s1.add(M, N, K, {mkterm(t.B, t.C, 1.0, 1.0)}, B_T, toff, M);
    toff += (long long)M * N;
    st2.push_back(mkterm(t.A, T, t.alpha[0], t.alpha[1]));
  }
  s2.add(orows, ocols, terms[0].A.ocols(), st2, obuf, ooff, orows);
}

static void build_tasks(pnfam_ctx* c) {
  const int nb = c->nb;
  const long long nxy = c->nxy;
  const int UL = c->left_u(), VL = c->left_v(), UR = c->right_u(), VR = c->right_v();
  auto X = [&](int i, int tr_) { return MatRef{B_STATE, c->xoff[i], c->db[i], c->db[c->xc[i]], tr_}; };
  auto Y = [&](int i, int tr_) { return MatRef{B_STATE, nxy + c->yoff[i], c->db[i], c->db[c->yc[i]], tr_}; };
  // statistical FAM: P and Q follow X and Y in the state (and in hqp)
  auto Pq = [&](int i, int tr_) { return MatRef{B_STATE, 2 * nxy + c->poff[i], c->db[i], c->db[c->pc[i]], tr_}; };
  auto Qq = [&](int i, int tr_) { return MatRef{B_STATE, 3 * nxy + c->qoff[i], c->db[i], c->db[c->qc[i]], tr_}; };
  const bool stat = c->nq == 4;
  c->k1a.clear(); c->k1b.clear(); c->k2a.clear(); c->k2b.clear();
  long long toff = 0;
  // ---- K1: dR_sp = W1 dR_qp W2^T (pnfam_solver.f90:144-150) ----
  // represented dR_qp = [P X; -Y -Q], W = [U V; V U]; stored quadrants of dR_sp
  // carry the signs and transposes of pnfam_solver.f90:357-363
  for (int i = 0; i < nb; ++i) {
    if (c->fc[i] < 0) continue;
    const int j = c->fc[i], x = c->xc[i], t = c->tr[i];
    // rho_pn = UL_i X_i VR_j^T - VL_i Y_t UR_j^T [+ UL_i P_i UR_j^T - VL_i Q_t VR_j^T]   (F structure, row i)
    std::vector<TripleTerm> r = {{{1.0, 1.0}, c->ublk(UL, i, 0), X(i, 0), c->vblk(VR, j, 1)},
                                 {{-1.0, -1.0}, c->vblk(VL, i, 0), Y(t, 0), c->ublk(UR, j, 1)}};
    if (stat) {
      r.push_back({{1.0, 1.0}, c->ublk(UL, i, 0), Pq(i, 0), c->ublk(UR, j, 1)});
      r.push_back({{-1.0, -1.0}, c->vblk(VL, i, 0), Qq(t, 0), c->vblk(VR, j, 1)});
    }
    emit_triple(c->k1a, c->k1b, toff, r, B_RSP, 0 * nxy + c->foff[i], c->db[i], c->db[j]);
    // kappa(+) stored = -UR_x X_i^T UL_i^T + VR_x Y_t^T VL_i^T [- VR_x P_i^T UL_i^T + UR_x Q_t^T VL_i^T]  (XT, row x)
    std::vector<TripleTerm> k = {{{-1.0, -1.0}, c->ublk(UR, x, 0), X(i, 1), c->ublk(UL, i, 1)},
                                 {{1.0, 1.0}, c->vblk(VR, x, 0), Y(t, 1), c->vblk(VL, i, 1)}};
    if (stat) {
      k.push_back({{-1.0, -1.0}, c->vblk(VR, x, 0), Pq(i, 1), c->ublk(UL, i, 1)});
      k.push_back({{1.0, 1.0}, c->ublk(UR, x, 0), Qq(t, 1), c->vblk(VL, i, 1)});
    }
    emit_triple(c->k1a, c->k1b, toff, k, B_RSP, 1 * nxy + c->xtoff[x], c->db[x], c->db[i]);
  }
  for (int i = 0; i < nb; ++i) {
    if (c->yc[i] < 0) continue;
    const int y = c->yc[i], t = c->tr[i];
    // kappa(-) stored = s (VR_y X_t^T VL_i^T - UR_y Y_i^T UL_i^T [+ UR_y P_t^T VL_i^T - VR_y Q_i^T UL_i^T]),
    // s = +1 Re, -1 Im  (YT, row y)
    std::vector<TripleTerm> k = {{{1.0, -1.0}, c->vblk(VR, y, 0), X(t, 1), c->vblk(VL, i, 1)},
                                 {{-1.0, 1.0}, c->ublk(UR, y, 0), Y(i, 1), c->ublk(UL, i, 1)}};
    if (stat) {
      k.push_back({{1.0, -1.0}, c->ublk(UR, y, 0), Pq(t, 1), c->vblk(VL, i, 1)});
      k.push_back({{-1.0, 1.0}, c->vblk(VR, y, 0), Qq(i, 1), c->ublk(UL, i, 1)});
    }
    emit_triple(c->k1a, c->k1b, toff, k, B_RSP, 2 * nxy + c->ytoff[y], c->db[y], c->db[i]);
  }
  for (int j = 0; j < nb; ++j) {
    if (c->fc[j] < 0) continue;
    const int i = c->fc[j], t = c->tr[i];
    // rho_np stored = -UR_j X_t^T VL_i^T + VR_j Y_i^T UL_i^T [- VR_j P_t^T VL_i^T + UR_j Q_i^T UL_i^T]  (F, row j)
    std::vector<TripleTerm> r = {{{-1.0, -1.0}, c->ublk(UR, j, 0), X(t, 1), c->vblk(VL, i, 1)},
                                 {{1.0, 1.0}, c->vblk(VR, j, 0), Y(i, 1), c->ublk(UL, i, 1)}};
    if (stat) {
      r.push_back({{-1.0, -1.0}, c->vblk(VR, j, 0), Pq(t, 1), c->vblk(VL, i, 1)});
      r.push_back({{1.0, 1.0}, c->ublk(UR, j, 0), Qq(i, 1), c->ublk(UL, i, 1)});
    }
    emit_triple(c->k1a, c->k1b, toff, r, B_RSP, 3 * nxy + c->foff[j], c->db[j], c->db[i]);
  }
  c->tplane = toff;
  // ---- K2: dH_qp = W1^T dH_sp W2 (pnfam_solver.f90:160-166) ----
  auto H = [&](int q, int row, const std::vector<long long>& off, const std::vector<int>& cols, int tr_) {
    return MatRef{B_HSP, q * nxy + off[row], c->db[row], c->db[cols[row]], tr_};
  };
  toff = 0;
  for (int i = 0; i < nb; ++i) {
    if (c->fc[i] < 0) continue;
    const int j = c->fc[i], x = c->xc[i], t = c->tr[i];
    // H20_i = UL_i^T h11_i VR_j + UL_i^T h12_i UR_x + s VL_t^T m21_t VR_j - VL_t^T m22_x^T UR_x
    emit_triple(c->k2a, c->k2b, toff,
                {{{1.0, 1.0}, c->ublk(UL, i, 1), H(0, i, c->foff, c->fc, 0), c->vblk(VR, j, 0)},
                 {{1.0, 1.0}, c->ublk(UL, i, 1), H(1, i, c->xoff, c->xc, 0), c->ublk(UR, x, 0)},
                 {{-1.0, 1.0}, c->vblk(VL, t, 1), H(2, t, c->yoff, c->yc, 0), c->vblk(VR, j, 0)},
                 {{-1.0, -1.0}, c->vblk(VL, t, 1), H(3, x, c->foff, c->fc, 1), c->ublk(UR, x, 0)}},
                B_HQP, c->xoff[i], c->db[i], c->db[x]);
  }
  for (int i = 0; i < nb; ++i) {
    if (c->yc[i] < 0) continue;
    const int y = c->yc[i], t = c->tr[i], j = c->xc[t];
    // H02s_i = -VL_t^T h11_t UR_y - s UL_i^T m21_i UR_y - VL_t^T h12_t VR_j + UL_i^T m22_j^T VR_j
    emit_triple(c->k2a, c->k2b, toff,
                {{{-1.0, -1.0}, c->vblk(VL, t, 1), H(0, t, c->foff, c->fc, 0), c->ublk(UR, y, 0)},
                 {{1.0, -1.0}, c->ublk(UL, i, 1), H(2, i, c->yoff, c->yc, 0), c->ublk(UR, y, 0)},
                 {{-1.0, -1.0}, c->vblk(VL, t, 1), H(1, t, c->xoff, c->xc, 0), c->vblk(VR, j, 0)},
                 {{1.0, 1.0}, c->ublk(UL, i, 1), H(3, j, c->foff, c->fc, 1), c->vblk(VR, j, 0)}},
                B_HQP, nxy + c->yoff[i], c->db[i], c->db[y]);
  }
  if (stat) {
    for (int i = 0; i < nb; ++i) {
      if (c->pc[i] < 0) continue;
      const int j = c->pc[i], x = c->xc[i], t = c->tr[i];
      // H11_i = UL_i^T h11_i UR_j + UL_i^T h12_i VR_x + s VL_t^T m21_t UR_j - VL_t^T m22_x^T VR_x
      emit_triple(c->k2a, c->k2b, toff,
                  {{{1.0, 1.0}, c->ublk(UL, i, 1), H(0, i, c->foff, c->fc, 0), c->ublk(UR, j, 0)},
                   {{1.0, 1.0}, c->ublk(UL, i, 1), H(1, i, c->xoff, c->xc, 0), c->vblk(VR, x, 0)},
                   {{-1.0, 1.0}, c->vblk(VL, t, 1), H(2, t, c->yoff, c->yc, 0), c->ublk(UR, j, 0)},
                   {{-1.0, -1.0}, c->vblk(VL, t, 1), H(3, x, c->foff, c->fc, 1), c->vblk(VR, x, 0)}},
                  B_HQP, 2 * nxy + c->poff[i], c->db[i], c->db[j]);
    }
    for (int i = 0; i < nb; ++i) {
      if (c->qc[i] < 0) continue;
      const int y = c->yc[i], q = c->qc[i], t = c->tr[i];
      // H11t_i = -VL_t^T h11_t VR_y - VL_t^T h12_t UR_q - s UL_i^T m21_i VR_y + UL_i^T m22_q^T UR_q
      emit_triple(c->k2a, c->k2b, toff,
                  {{{-1.0, -1.0}, c->vblk(VL, t, 1), H(0, t, c->foff, c->fc, 0), c->vblk(VR, y, 0)},
                   {{-1.0, -1.0}, c->vblk(VL, t, 1), H(1, t, c->xoff, c->xc, 0), c->ublk(UR, q, 0)},
                   {{1.0, -1.0}, c->ublk(UL, i, 1), H(2, i, c->yoff, c->yc, 0), c->vblk(VR, y, 0)},
                   {{1.0, 1.0}, c->ublk(UL, i, 1), H(3, q, c->foff, c->fc, 1), c->ublk(UR, q, 0)}},
                  B_HQP, 3 * nxy + c->qoff[i], c->db[i], c->db[q]);
    }
  }
  c->tplane = std::max(c->tplane, toff);
  // ---- FP64 field projection tasks: spin-uniform tiles of 1024 / tn rows x tn columns ----
  // The shape of each (block pair, spin segment) is the one that issues the fewest DFMAs:
  // per tile, tn columns x the rows up to the warp granularity of the shape (a warp holds
  // 64 / (tn / 2) rows and skips when they are all beyond the tile), twice (Re, Im), plus
  // the hpsi generation (10 DFMAs per column and mesh point of each component)
  c->htasks.clear();
  auto cdiv = [](int a, int b) { return (a + b - 1) / b; };
  auto add_h = [&](int ix, int iy, int mode, int call, int outq, long long ooff) {
    const int d = c->db[ix], dc = c->db[iy], nu = c->nup[ix];
    const int seg[3] = {0, nu, d};
    for (int s = 0; s < 2; ++s) {
      const int n = seg[s + 1] - seg[s];
      if (n <= 0) continue;
      int best = 32;
      long long bcost = -1;
      for (int tn : {32, 16, 8}) {
        const int tm = 1024 / tn, wr = 128 / tn;   // rows per tile, rows per warp
        long long cost = 0;
        for (int a0 = 0; a0 < n; a0 += tm) {
          const int na = std::min(tm, n - a0);
          cost += (long long)cdiv(dc, tn) * tn * (2LL * cdiv(na, wr) * wr + 10);
        }
        if (bcost < 0 || cost < bcost) { bcost = cost; best = tn; }
      }
      const int tm = 1024 / best;
      for (int a0 = seg[s]; a0 < seg[s + 1]; a0 += tm)
        for (int b0 = 0; b0 < dc; b0 += best) {
          HTask h{};
          h.ix = ix; h.iy = iy; h.a0 = a0; h.na = std::min(tm, seg[s + 1] - a0);
          h.b0 = b0; h.nbc = std::min(best, dc - b0); h.sa = s == 0 ? 1 : -1;
          h.mode = mode; h.call = call; h.outq = outq; h.tn = best; h.ooff = ooff;
          c->htasks.push_back(h);
        }
    }
  };
  // tensor-core tiles: rows of the output block (N <= 128, padded to 16) against up to
  // 64 columns x pg points (M = 128 = Re and Im of 64 hpsi rows)
  c->htasks_tc.clear();
  c->tc_npmax = 16;
  auto add_tc = [&](int ix, int iy, int mode, int call, int outq, long long ooff) {
    const int d = c->db[ix], dc = c->db[iy], nu = c->nup[ix];
    const int seg[3] = {0, nu, d};
    for (int s = 0; s < 2; ++s) {
      const int nseg = seg[s + 1] - seg[s];
      if (nseg <= 0) continue;
      const int wa = cdiv(nseg, cdiv(nseg, (int)HTC_MAXN));
      for (int a0 = seg[s]; a0 < seg[s + 1]; a0 += wa) {
        const int na = std::min(wa, seg[s + 1] - a0);
        const int wb = cdiv(dc, cdiv(dc, (int)HTC_MAXB));
        for (int b0 = 0; b0 < dc; b0 += wb) {
          HTaskTC h;
          h.ix = ix; h.iy = iy; h.a0 = a0; h.na = na; h.b0 = b0; h.nbc = std::min(wb, dc - b0);
          h.sa = s == 0 ? 1 : -1; h.mode = mode; h.call = call; h.outq = outq; h.ooff = ooff;
          h.np = std::max(16, cdiv(na, 16) * 16);
          h.pg = std::max(1, std::min<int>(HTC_MAXPG, HTC_MAXB / h.nbc));
          c->htasks_tc.push_back(h);
          c->tc_npmax = std::max(c->tc_npmax, h.np);
        }
      }
    }
  };
  for (int i = 0; i < nb; ++i) {
    if (c->fc[i] >= 0) { add_h(i, c->fc[i], 0, 0, 0, c->foff[i]); add_h(i, c->fc[i], 0, 1, 3, c->foff[i]); }
    if (c->xc[i] >= 0) add_h(i, c->xc[i], 1, 0, 1, c->xoff[i]);
    if (c->yc[i] >= 0) add_h(i, c->yc[i], 1, 1, 2, c->yoff[i]);
    if (c->fc[i] >= 0) { add_tc(i, c->fc[i], 0, 0, 0, c->foff[i]); add_tc(i, c->fc[i], 0, 1, 3, c->foff[i]); }
    if (c->xc[i] >= 0) add_tc(i, c->xc[i], 1, 0, 1, c->xoff[i]);
    if (c->yc[i] >= 0) add_tc(i, c->yc[i], 1, 1, 2, c->yoff[i]);
  }
  // pre-split row basis functions of the projection tiles, one copy per distinct
  // (block, first row, rows)
  c->hptiles.clear();
  {
    const long long nrc = (c->nghl + HTC_K - 1) / HTC_K;
    std::map<std::tuple<int, int, int>, long long> seen;
    long long off = 0;
    for (HTaskTC& h : c->htasks_tc) {
      const auto key = std::make_tuple(h.ix, h.a0, h.na);
      auto it = seen.find(key);
      if (it == seen.end()) {
        it = seen.emplace(key, off).first;
        c->hptiles.push_back(HPTile{h.ix, h.a0, h.na, h.np, off});
        off += 5 * nrc * 64 * (long long)h.np;
      }
      h.tphi = it->second;
    }
    c->hphi_floats = off;
    c->have_hphi = false;
  }
  // tensor-core densities: A chunks per (block, spin of the rows, 8 rows); units per
  // call in the order (kind, ix, column range, spin), so that the two spins of one
  // column range follow each other; B chunks with their place in a point's buffer
  c->achunks.clear();
  std::vector<int> aidx(2 * nb, 0);
  for (int i = 0; i < nb; ++i) {
    const int seg[3] = {0, c->nup[i], c->db[i]};
    for (int s = 0; s < 2; ++s) {
      aidx[2 * i + s] = (int)c->achunks.size();
      for (int a0 = seg[s]; a0 < seg[s + 1]; a0 += 8) c->achunks.push_back(DAChunkTC{i, a0, seg[s + 1], 0});
    }
  }
  c->bchunks.clear();
  long long boff = 0;
  for (int call = 0; call < 2; ++call) {
    auto& U = c->dunits[call];
    U.clear();
    for (int kind = 0; kind < 2; ++kind) {
      const std::vector<int>& cols = kind == 0 ? c->fc : (call == 0 ? c->xtc : c->ytc);
      for (int ix = 0; ix < nb; ++ix) {
        const int iy = cols[ix];
        if (iy < 0) continue;
        const int dc = c->db[iy];
        const int nh = cdiv(dc, (int)DTC2_MAXNC), csz = cdiv(dc, nh);
        const int seg[3] = {0, c->nup[ix], c->db[ix]};
        for (int b0 = 0; b0 < dc; b0 += csz) {
          const int nc = std::min(csz, dc - b0), npad = cdiv(2 * nc, 16) * 16;
          for (int s = 0; s < 2; ++s) {
            if (seg[s] >= seg[s + 1]) continue;
            DUnitTC u;
            u.kind = kind; u.ix = ix; u.iy = iy; u.s = s; u.b0 = b0; u.nc = nc; u.npad = npad;
            u.nk = cdiv(seg[s + 1] - seg[s], 8); u.achunk = aidx[2 * ix + s]; u.nub = c->nup[iy]; u.boff = boff;
            for (int kc = 0; kc < u.nk; ++kc) {
              c->bchunks.push_back(DBChunkTC{call, kind, ix, seg[s] + 8 * kc, seg[s + 1], b0, nc, npad,
                                             boff + (long long)kc * 16 * npad});
            }
            boff += (long long)u.nk * 16 * npad;
            U.push_back(u);
          }
        }
      }
    }
  }
  c->bstride = (boff + 63) / 64 * 64;
}

// ---------------------------------------------------------------------------
// buffers for a batch of P points
// ---------------------------------------------------------------------------
// live kernel timing: the event index of a launch about to be enqueued on st (-1 when
// live timing is off or an event could not be made)
static int live_begin(pnfam_ctx* c, cudaStream_t st) {
  if (!c->live) return -1;
  while ((int)c->lev.size() < c->nlev + 2) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return -1;
    c->lev.push_back(e);
  }
  const int i = c->nlev;
  if (cudaEventRecord(c->lev[i], st) != cudaSuccess) return -1;
  c->nlev += 2;
  c->lkind.resize(c->nlev / 2);
  c->lkind[i / 2] = -1;
  return i;
}

static void live_end(pnfam_ctx* c, int i, int kind, cudaStream_t st) {
  if (i < 0) return;
  if (cudaEventRecord(c->lev[i + 1], st) == cudaSuccess) c->lkind[i / 2] = kind;
}

// after the stream of the timed launches has been waited for
static void live_collect(pnfam_ctx* c) {
  for (int i = 0; i + 1 < c->nlev; i += 2) {
    const int k = c->lkind[i / 2];
    float ms = 0.f;
    if (k >= 0 && cudaEventElapsedTime(&ms, c->lev[i], c->lev[i + 1]) == cudaSuccess) {
      c->live_ms[k] += ms;
      c->live_n[k] += 1;
    }
  }
  c->nlev = 0;
}

// ---------------------------------------------------------------------------
// pair-tensor GEMMs (pair_gemm.cuh): problems, element lists, tasks
// ---------------------------------------------------------------------------
// dynamic shared memory of k_pg_gemm: by default 104 KB (pnfam_ctx::pg_smem), so that
// two of its CTAs share an SM and one streams while the other starts or drains a task;
// at most PG_SMEM_MAX
static constexpr int PG_SMEM_MAX = 224 * 1024;

// stages of k_pg_gemm for B slots of bslot floats
static int pg_stages(int bslot, int smem) {
  const int per = (int)((PG_ACHUNK + bslot) * sizeof(float));
  return std::max(2, std::min((int)PG_MAXSTAGE, smem / per));
}

// K chunks per density task the autotuner tries (the finest first)
static constexpr int PG_KSPANS[4] = {96, 192, 384, 768};

// density tasks (problem, M tile, K range of at most kspan chunks) and the layout of
// their partial sums; the largest tasks first
static void pg_density_tasks(pnfam_ctx* c, int kspan) {
  auto cdiv = [](long long a, long long b) { return (a + b - 1) / b; };
  c->pg_tdens.clear();
  long long d0 = 0;
  for (int id = 0; id < (int)c->pg_probs.size(); ++id) {
    PGProb& pr = c->pg_probs[id];
    if (pr.kind != 1) continue;
    pr.nsplit = (int)std::max(1LL, cdiv(pr.nkc, kspan));
    pr.d0 = d0;
    d0 += (long long)pr.nsplit * pr.ncol * PG_MAXPTS * pr.mrows;
    for (int t = 0; t < pr.ntile; ++t)
      for (int sp = 0; sp < pr.nsplit; ++sp) {
        const int k0 = (int)((long long)pr.nkc * sp / pr.nsplit), k1 = (int)((long long)pr.nkc * (sp + 1) / pr.nsplit);
        if (k1 <= k0) continue;
        c->pg_tdens.push_back(PGTask{id, t, k0, k1 - k0, sp, 0});
      }
  }
  std::stable_sort(c->pg_tdens.begin(), c->pg_tdens.end(),
                   [](const PGTask& x, const PGTask& y) { return x.nkc > y.nkc; });
  c->pg_dfloats = d0;
  c->pg_kspan = kspan;
}

static void pg_setup(pnfam_ctx* c) {
  c->pg_on = false;
  c->pg_built = false;
  c->pg_probs.clear(); c->pg_elems.clear(); c->pg_tproj.clear(); c->pg_tdens.clear();
  c->pg_bproj.clear(); c->pg_bdens.clear(); c->pg_ach.clear();
  for (int k = 0; k < 12; ++k) c->pg_fold.dens[k] = -1;
  if (!c->pg_mode) return;
  const int nghl = c->nghl, nb = c->nb;
  auto cdiv = [](long long a, long long b) { return (a + b - 1) / b; };
  // element lists of one structure, per class, in (block row, column, row) order
  auto elements = [&](const std::vector<int>& cols, const std::vector<long long>& offs,
                      std::vector<PGElem> (&out)[4]) {
    for (int ix = 0; ix < nb; ++ix) {
      const int iy = cols[ix];
      if (iy < 0) continue;
      const int d = c->db[ix], dc = c->db[iy];
      for (int b = 0; b < dc; ++b)
        for (int a = 0; a < d; ++a) {
          const int ja = c->st[ix] + a, jb = c->st[iy] + b;
          const int k = 2 * (c->ns[ja] < 0) + (c->ns[jb] < 0);
          out[k].push_back(PGElem{ja, jb, offs[ix] + a + (long long)b * d});
        }
    }
  };
  long long a0 = 0, b0 = 0, d0 = 0;
  auto add = [&](int kind, int pairing, int ncombo, int cls, int ncol, int call, const std::vector<PGElem>& el) {
    if (el.empty()) return -1;
    PGProb pr{};
    pr.kind = kind; pr.pairing = pairing; pr.ncombo = ncombo; pr.cls = cls; pr.ncol = ncol; pr.call = call;
    pr.e0 = (long long)c->pg_elems.size(); pr.ne = (int)el.size();
    c->pg_elems.insert(c->pg_elems.end(), el.begin(), el.end());
    if (kind == 0) { pr.mrows = pr.ne; pr.kdim = ncombo * nghl; }
    else { pr.mrows = ncombo * nghl; pr.kdim = pr.ne; }
    pr.nkc = (int)cdiv(pr.kdim, PG_K);
    pr.ntile = (int)cdiv(pr.mrows, PG_M);
    pr.nsplit = 1;   // density problems: pg_density_tasks
    pr.a0 = a0; a0 += (long long)pr.ntile * pr.nkc;
    pr.b0 = b0; b0 += pr.nkc;
    pr.d0 = 0;
    const int id = (int)c->pg_probs.size();
    c->pg_probs.push_back(pr);
    if (kind == 0)
      for (int t = 0; t < pr.ntile; ++t) c->pg_tproj.push_back(PGTask{id, t, 0, pr.nkc, 0, 0});
    for (int kc = 0; kc < pr.nkc; ++kc) (kind == 0 ? c->pg_bproj : c->pg_bdens).push_back(PGBChunk{id, kc});
    return id;
  };
  std::vector<PGElem> ef[4], ex[4], ey[4], ext[4], eyt[4];
  elements(c->fc, c->foff, ef);
  elements(c->xc, c->xoff, ex);
  elements(c->yc, c->yoff, ey);
  elements(c->xtc, c->xtoff, ext);
  elements(c->ytc, c->ytoff, eyt);
  for (int k = 0; k < 4; ++k) {
    add(0, 0, 18, k, 4, -1, ef[k]);
    add(0, 1, 1, k, 2, 0, ex[k]);
    add(0, 1, 1, k, 2, 1, ey[k]);
    c->pg_fold.dens[k] = add(1, 0, 16, k, 4, -1, ef[k]);
    c->pg_fold.dens[4 + k] = add(1, 1, 1, k, 2, 0, ext[k]);
    c->pg_fold.dens[8 + k] = add(1, 1, 1, k, 2, 1, eyt[k]);
  }
  c->pg_nachunk = a0;
  c->pg_nbchunk = b0;
  c->pg_tuned = false;
  c->pg_kspan = c->pg_kspan_env > 0 ? c->pg_kspan_env : 384;
  pg_density_tasks(c, c->pg_kspan);
  // the largest tasks first: the long projection tiles
  std::stable_sort(c->pg_tproj.begin(), c->pg_tproj.end(),
                   [](const PGTask& x, const PGTask& y) { return x.nkc > y.nkc; });
  // budget with the partial sums of the finest density split the autotuner may choose
  long long dmax = 0;
  for (const PGProb& pr : c->pg_probs)
    if (pr.kind == 1) dmax += (long long)std::max(1LL, cdiv(pr.nkc, PG_KSPANS[0])) * pr.ncol * PG_MAXPTS * pr.mrows;
  (void)d0;
  const double bytes = (double)a0 * PG_ACHUNK * sizeof(float) + (double)b0 * PG_BCHUNK * sizeof(float) +
                       (double)dmax * sizeof(float);
  c->pg_on = bytes <= c->pg_budget;
  if (!c->pg_on) return;
  for (int id = 0; id < (int)c->pg_probs.size(); ++id) {
    const PGProb& pr = c->pg_probs[id];
    for (int t = 0; t < pr.ntile; ++t)
      for (int kc = 0; kc < pr.nkc; ++kc) c->pg_ach.push_back(PGAChunk{id, t, kc, 0});
  }
}

// device tables and the pair tensor (once per operator)
static int pg_build(pnfam_ctx* c) {
  if (!c->pg_on || c->pg_built) return PNFAM_OK;
  CK(upload(c->d_pg_probs, c->pg_probs.data(), c->pg_probs.size()));
  CK(upload(c->d_pg_elems, c->pg_elems.data(), c->pg_elems.size()));
  CK(upload(c->d_pg_tproj, c->pg_tproj.data(), c->pg_tproj.size()));
  CK(upload(c->d_pg_tdens, c->pg_tdens.data(), c->pg_tdens.size()));
  CK(upload(c->d_pg_bproj, c->pg_bproj.data(), c->pg_bproj.size()));
  CK(upload(c->d_pg_bdens, c->pg_bdens.data(), c->pg_bdens.size()));
  CK(dalloc(c->d_pg_a, (size_t)c->pg_nachunk * PG_ACHUNK));
  CK(dalloc(c->d_pg_b, (size_t)c->pg_nbchunk * PG_BCHUNK));
  CK(dalloc(c->d_pg_d, (size_t)std::max(1LL, c->pg_dfloats)));
  DBuf<PGAChunk> d_ach;
  const cudaError_t e = upload(d_ach, c->pg_ach.data(), c->pg_ach.size());
  if (e != cudaSuccess) { d_ach.release(); CK(e); }
  const long long n = (long long)c->pg_ach.size();
  for (long long i0 = 0; i0 < n; i0 += 1 << 20) {
    const unsigned g = (unsigned)std::min<long long>(1 << 20, n - i0);
    k_pg_build<<<g, 256, 0, c->stream>>>(c->d_phi32.p, c->dqp, c->nghl, c->d_pg_probs.p, c->d_pg_elems.p,
                                         d_ach.p + i0, c->d_pg_a.p);
  }
  const cudaError_t le = cudaGetLastError();
  const cudaError_t se = cudaStreamSynchronize(c->stream);
  d_ach.release();
  CK(le);
  CK(se);
  std::vector<PGAChunk>().swap(c->pg_ach);
  c->pg_built = true;
  return PNFAM_OK;
}

// densities of the points in c->d_actlist (nact of them) into dpart [P][2][1][2 ND][nghl]
static int pg_density(pnfam_ctx* c, int nact, const float* rsp, float* dpart, cudaStream_t st) {
  for (int g0 = 0; g0 < nact; g0 += PG_MAXPTS) {
    const int na = std::min((int)PG_MAXPTS, nact - g0);
    const int* al = c->d_actlist.p + g0;
    const int bslot = ((4 * na + 15) / 16 * 16) * PG_K * 2;
    const int ns = pg_stages(bslot, c->pg_smem);
    k_pg_pack_rho<<<(unsigned)c->pg_bdens.size(), 256, 0, st>>>(c->d_pg_probs.p, c->d_pg_elems.p, c->d_pg_bdens.p,
                                                                 al, na, rsp, c->nxy, c->d_pg_b.p);
    const int lv = live_begin(c, st);
    k_pg_gemm<<<(unsigned)c->pg_tdens.size(), PG_THREADS, pg_smem_bytes(ns, bslot), st>>>(
        c->d_pg_probs.p, c->d_pg_tdens.p, c->d_pg_elems.p, c->d_pg_a.p, c->d_pg_b.p, na, al, ns, bslot, nullptr,
        c->nxy, c->d_pg_d.p, c->d_err.p);
    live_end(c, lv, 0, st);
    k_pg_fold<<<dim3((unsigned)((c->nghl + PG_FOLD_R - 1) / PG_FOLD_R), (unsigned)na, 2), 4 * PG_FOLD_R, 0, st>>>(
        c->d_pg_probs.p, c->pg_fold, c->d_pg_d.p, al, c->nghl, dpart);
    c->launches += 3;
    CK(cudaGetLastError());
  }
  return PNFAM_OK;
}

// field projection of the points in c->d_actlist into hsp [P][2][4][nxy]
static int pg_projection(pnfam_ctx* c, int nact, const float* mf, float* hsp, cudaStream_t st) {
  for (int g0 = 0; g0 < nact; g0 += PG_MAXPTS) {
    const int na = std::min((int)PG_MAXPTS, nact - g0);
    const int* al = c->d_actlist.p + g0;
    const int bslot = ((4 * na + 15) / 16 * 16) * PG_K * 2;
    const int ns = pg_stages(bslot, c->pg_smem);
    k_pg_pack_field<<<(unsigned)c->pg_bproj.size(), 256, 0, st>>>(c->d_pg_probs.p, c->d_pg_bproj.p, al, na, mf,
                                                                   c->nghl, c->d_pg_b.p);
    const int lv = live_begin(c, st);
    k_pg_gemm<<<(unsigned)c->pg_tproj.size(), PG_THREADS, pg_smem_bytes(ns, bslot), st>>>(
        c->d_pg_probs.p, c->d_pg_tproj.p, c->d_pg_elems.p, c->d_pg_a.p, c->d_pg_b.p, na, al, ns, bslot, hsp,
        c->nxy, nullptr, c->d_err.p);
    live_end(c, lv, 1, st);
    c->launches += 2;
    CK(cudaGetLastError());
  }
  return PNFAM_OK;
}

static int ensure_buffers(pnfam_ctx* c, int P, int M) {
  const long long nxy = c->nxy;
  const long long nv = 2 * c->nq * nxy;   // Re and Im of the QP state (X, Y[, P, Q])
  const long long tpl = std::max(c->tplane, 8 * nxy);
  CK(dalloc(c->d_state, (size_t)P * nv));
  CK(dalloc(c->d_vout, (size_t)P * nv));
  CK(dalloc(c->d_T, (size_t)P * 2 * tpl));
  CK(dalloc(c->d_rsp, (size_t)P * 8 * nxy));
  CK(dalloc(c->d_hsp, (size_t)P * 8 * nxy));
  CK(dalloc(c->d_hqp, (size_t)P * nv));
  CK(dalloc(c->d_dpart, (size_t)P * 2 * c->G * 2 * ND * c->nghl));
  CK(dalloc(c->d_mf, (size_t)P * 2 * NMF * 2 * c->nghl));
  const int Mh = std::max(M, 1);
  CK(dalloc(c->d_df, (size_t)P * Mh * nv));
  CK(dalloc(c->d_dv, (size_t)P * Mh * nv));
  CK(dalloc(c->d_bpart, (size_t)P * c->nchunk_bro * BRO_NPART));
  CK(dalloc(c->d_si, (size_t)P));
  CK(dalloc(c->d_norm, (size_t)P));
  CK(dalloc(c->d_beta, (size_t)P * Mh * Mh));
  CK(dalloc(c->d_gamma, (size_t)P * 64));
  CK(dalloc(c->d_cpart, (size_t)P * c->nchunk_c * 2 * c->nops));
  CK(dalloc(c->d_wre, (size_t)P));
  CK(dalloc(c->d_wim, (size_t)P));
  CK(dalloc(c->d_gfn, (size_t)P * nv));
  CK(dalloc(c->d_active, (size_t)P));
  CK(dalloc(c->d_pint, (size_t)6 * P));
  CK(dalloc(c->d_actlist, (size_t)P));
  if (!c->d_err.p) {
    CK(dalloc(c->d_err, 1));
    CK(cudaMemsetAsync(c->d_err.p, 0, sizeof(int), c->stream));
  }
  CK(dalloc(c->d_act32, (size_t)P));
  CK(dalloc(c->d_act64, (size_t)P));
  CK(dalloc(c->d_act64r, (size_t)ANCH_RING * P));
  BufDesc bd[NBUF];
  bd[B_UP] = {c->d_up.p, 0, 0};
  bd[B_VP] = {c->d_vp.p, 0, 0};
  bd[B_UN] = {c->d_un.p, 0, 0};
  bd[B_VN] = {c->d_vn.p, 0, 0};
  bd[B_STATE] = {c->d_state.p, nv, nv / 2};
  bd[B_T] = {c->d_T.p, 2 * tpl, tpl};
  bd[B_RSP] = {c->d_rsp.p, 8 * nxy, 4 * nxy};
  bd[B_HSP] = {c->d_hsp.p, 8 * nxy, 4 * nxy};
  bd[B_HQP] = {c->d_hqp.p, nv, nv / 2};
  CK(upload(c->d_bufs, bd, NBUF));
  return PNFAM_OK;
}

template <class T>
static int launch_gemm(pnfam_ctx* c, TaskList& tl, int P, const int* active, const BufDescT<T>* bufs,
                       cudaStream_t st) {
  if (tl.ntiles == 0) return PNFAM_OK;
  dim3 grid(tl.ntiles, 2 * P);
  k_gemm<T><<<grid, 256, 0, st>>>(tl.d_tasks.p, tl.d_tile2task.p, bufs, active);
  c->launches++;
  CK(cudaGetLastError());
  return PNFAM_OK;
}

// FP32 stage on the tensor cores for the nact points listed in c->d_actlist
static int launch_gemm_tc(pnfam_ctx* c, TaskListTC& tl, int nact, cudaStream_t st) {
  if (tl.tasks.empty() || nact <= 0) return PNFAM_OK;
  dim3 grid((unsigned)tl.tasks.size(), (unsigned)((2 * nact * tl.maxrows + 127) / 128));
  k_gemm_tc<<<grid, GTC_THREADS, gemm_tc_smem_bytes(tl.maxnp), st>>>(tl.d_tasks.p, c->d_bufs32.p, c->d_gsplit.p,
                                                                      c->d_actlist.p, nact, tl.maxnp, c->d_err.p);
  c->launches++;
  CK(cudaGetLastError());
  return PNFAM_OK;
}

static int launch_gemm(pnfam_ctx* c, TaskList& tl, int P, const int* active) {
  return launch_gemm<double>(c, tl, P, active, c->d_bufs.p, c->stream);
}

// residual interaction of the points flagged in `act`: state (X, Y[, P, Q]) -> hqp
// (H20, H02[, H11, H11t] stored), computed in precision T (the FP32 form reads the FP32
// copy of the state and writes the FP32 hqp)
template <class T>
// P: batch size (grid extent), nact: points active in this evaluation
static int residual_t(pnfam_ctx* c, int P, int nact, const int* act, bool timed, cudaStream_t st) {
  auto tic = [&]() { if (timed) cudaEventRecord(c->ev[0], st); };
  auto toc = [&](int k) {
    if (!timed) return;
    cudaEventRecord(c->ev[1], st);
    cudaEventSynchronize(c->ev[1]);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
    (std::is_same<T, float>::value ? c->stage32_ms : c->stage_ms)[k] += ms;
  };
  constexpr bool f32 = std::is_same<T, float>::value;
  const BufDescT<T>* bufs;
  T *rsp, *hsp, *dpart, *mf;
  if constexpr (f32) {
    bufs = c->d_bufs32.p; rsp = c->d_rsp32.p; hsp = c->d_hsp32.p; dpart = c->d_dpart32.p; mf = c->d_mf32.p;
  } else {
    bufs = c->d_bufs.p; rsp = c->d_rsp.p; hsp = c->d_hsp.p; dpart = c->d_dpart.p; mf = c->d_mf.p;
  }
  int rc;
  tic();
  if constexpr (f32) {
    if ((rc = launch_gemm_tc(c, c->t1a, nact, st))) return rc;
    if ((rc = launch_gemm_tc(c, c->t1b, nact, st))) return rc;
  } else {
    if ((rc = launch_gemm<T>(c, c->k1a, P, act, bufs, st))) return rc;
    if ((rc = launch_gemm<T>(c, c->k1b, P, act, bufs, st))) return rc;
  }
  toc(0);
  const long long nxy = c->nxy;
  DensCallT<T> d0, d1;
  d0.rho = rsp + 0 * nxy; d0.rho_sp = 8 * nxy; d0.rho_spl = 4 * nxy;
  d0.rcols = c->d_fc.p; d0.roffs = c->d_foff.p;
  d0.kap = rsp + 1 * nxy; d0.kap_sp = 8 * nxy; d0.kap_spl = 4 * nxy;
  d0.kcols = c->d_xtc.p; d0.koffs = c->d_xtoff.p;
  d1.rho = rsp + 3 * nxy; d1.rho_sp = 8 * nxy; d1.rho_spl = 4 * nxy;
  d1.rcols = c->d_fc.p; d1.roffs = c->d_foff.p;
  d1.kap = rsp + 2 * nxy; d1.kap_sp = 8 * nxy; d1.kap_spl = 4 * nxy;
  d1.kcols = c->d_ytc.p; d1.koffs = c->d_ytoff.p;
  const DevBasisT<T> B = c->devbasis<T>();
  // block-row groups: FP32, enough CTAs to fill the GPU twice over for the active
  // points; FP64, always the context's group count, so that a point's sums (and its
  // result) do not depend on which other points share the evaluation
  const int ntr = (c->nghl + DRT - 1) / DRT;
  const int na = std::max(nact, 1);
  const int G = f32 ? std::max(1, std::min(c->G, (2 * c->nsm + ntr * 2 * na - 1) / (ntr * 2 * na))) : c->G;
  int Gm = G;   // block-row groups of the partial densities
  bool dens_done = false;
  // pair-tensor GEMMs for evaluations of enough points (one partial group)
  const bool pair = f32 && c->pg_on && c->pg_built && nact >= c->pg_min;
  tic();
  if constexpr (f32) {
    if (pair) {
      if ((rc = pg_density(c, nact, rsp, dpart, st))) return rc;
      Gm = 1;
      dens_done = true;
    } else if (c->tc_density) {
      // tensor cores: c->d_actlist holds the nact points of this evaluation; their
      // densities are split and laid out first, then the units run on the tensor cores
      DensTCArgs t0{d0.rho, d0.rho_sp, d0.rho_spl, d0.rcols, d0.roffs, d0.kap, d0.kap_sp, d0.kap_spl, d0.kcols, d0.koffs};
      DensTCArgs t1{d1.rho, d1.rho_sp, d1.rho_spl, d1.rcols, d1.roffs, d1.kap, d1.kap_sp, d1.kap_spl, d1.kcols, d1.koffs};
      const int ntr32 = (c->nghl + 31) / 32;
      Gm = std::max(1, std::min(c->G, (2 * c->nsm + ntr32 * 2 * na - 1) / (ntr32 * 2 * na)));
      const int lv = live_begin(c, st);
      if (!c->bchunks.empty()) {
        k_dens_bsplit<<<dim3((unsigned)c->bchunks.size(), (unsigned)na), 256, 0, st>>>(
            B, t0, t1, c->d_bchunks.p, c->d_actlist.p, c->d_bsplit.p, c->bstride);
        c->launches++;
      }
      k_density_tc2<<<dim3(ntr32, Gm, 2 * na), DTC2_THREADS, density_tc2_smem_bytes(), st>>>(
          B, c->d_dunits0.p, (int)c->dunits[0].size(), c->d_dunits1.p, (int)c->dunits[1].size(), c->d_aphi.p,
          (int)c->achunks.size(), c->d_bsplit.p, c->bstride, Gm, c->d_actlist.p, dpart, c->d_err.p);
      live_end(c, lv, 0, st);
      c->launches++;
      CK(cudaGetLastError());
      dens_done = true;
    }
  }
  if (!dens_done) {
    dim3 grid(ntr, G, 2 * P);
    if constexpr (f32) k_density<float><<<grid, 256, density_smem_bytes<float>(), st>>>(B, d0, d1, G, dpart, act);
    else k_density_fp64<<<grid, 256, 0, st>>>(B, d0, d1, G, dpart, act);
    c->launches++;
    CK(cudaGetLastError());
  }
  toc(1);
  tic();
  {
    dim3 grid((c->nghl + 127) / 128, 2 * P);
    k_meanfield<T><<<grid, 128, 0, st>>>(B, Gm, dpart, mf, act);
    c->launches++;
    CK(cudaGetLastError());
  }
  toc(2);
  tic();
  if constexpr (f32) {
    if (pair) {
      if ((rc = pg_projection(c, nact, mf, hsp, st))) return rc;
    } else {
      // tensor cores: c->d_actlist holds the nact points of this evaluation
      dim3 grid((unsigned)c->htasks_tc.size(), (unsigned)std::max(nact, 1));
      const int lv = live_begin(c, st);
      k_hproj_tc<<<grid, HTC_THREADS, hproj_tc_smem_bytes(c->tc_npmax), st>>>(
          B, c->d_htasks_tc.p, c->d_actlist.p, nact, c->tc_npmax, mf, c->d_hphi.p, hsp, nxy, c->d_err.p);
      live_end(c, lv, 1, st);
      c->launches++;
      CK(cudaGetLastError());
    }
  } else {
    dim3 grid((unsigned)c->htasks.size(), P);
    k_hproj_fp64<<<grid, 256, hproj_fp64_smem_bytes(), st>>>(B, c->d_htasks.p, mf, hsp, nxy, act);
    c->launches++;
    CK(cudaGetLastError());
  }
  toc(3);
  tic();
  if constexpr (f32) {
    if ((rc = launch_gemm_tc(c, c->t2a, nact, st))) return rc;
    if ((rc = launch_gemm_tc(c, c->t2b, nact, st))) return rc;
  } else {
    if ((rc = launch_gemm<T>(c, c->k2a, P, act, bufs, st))) return rc;
    if ((rc = launch_gemm<T>(c, c->k2b, P, act, bufs, st))) return rc;
  }
  toc(4);
  return PNFAM_OK;
}


// ---------------------------------------------------------------------------
// Autotuning of the FP32 evaluation, once per operator (after its pair tensor is
// built), from the operator's block structure and timed trial evaluations:
//  1. the K span of the density tasks of the pair-tensor GEMM.  The problem sizes
//     (rows = component pairs x mesh points, K = the elements of a spin class, both
//     fixed by the block-size histogram) give the task count of each candidate span,
//     hence its number of waves on the SMs; the candidates whose last wave is at least
//     half full, or the finest one, are timed and the fastest is kept.
//  2. pg_min, the point count from which an evaluation takes the pair-tensor path
//     instead of the per-block tensor-core kernels: both are timed at 1, 2, 4, ... up
//     to 64 points (or the engine's slots) and pg_min is the smallest count from which
//     the pair path stays the faster one (PNFAM_GB300_PAIR_MIN fixes it instead).
// Trial evaluations run on the FP32 scratch of the context's first slots (zeroed), on
// the context's stream, before any point is admitted.  PNFAM_GB300_AUTOTUNE=0 skips it.
// ---------------------------------------------------------------------------
// Choices are kept per process, keyed by what they depend on (the problem sizes of
// the operator's pair tensor, the mesh, the trial point count, the SM count), so a
// later context of the same operator structure takes them without trials.
struct TuneChoice { int kspan, pg_min; };
static std::mutex g_tune_mu;
static std::map<unsigned long long, TuneChoice> g_tune;

static unsigned long long pg_tune_key(const pnfam_ctx* c, int nmax) {
  unsigned long long h = 1469598103934665603ULL;
  auto mix = [&](long long v) {
    for (int b = 0; b < 8; ++b) { h ^= (unsigned long long)((v >> (8 * b)) & 0xff); h *= 1099511628211ULL; }
  };
  mix(c->nghl); mix(c->nq); mix(nmax); mix(c->nsm); mix(c->dev); mix(c->pg_min_env ? c->pg_min : -1);
  mix(c->pg_kspan_env); mix(c->pg_smem);
  for (const PGProb& pr : c->pg_probs) { mix(pr.kind); mix(pr.ntile); mix(pr.nkc); mix(pr.ncol); }
  return h;
}

static int pg_autotune(pnfam_ctx* c, int P) {
  const int nmax = std::min(P, (int)PG_MAXPTS);
  if (c->pg_tuned || !c->pg_on || !c->pg_built || !c->autotune || nmax < 2) return PNFAM_OK;
  c->pg_tuned = true;
  const unsigned long long key = pg_tune_key(c, nmax);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      if (it->second.kspan != c->pg_kspan) {
        pg_density_tasks(c, it->second.kspan);
        CK(upload(c->d_pg_probs, c->pg_probs.data(), c->pg_probs.size()));
        CK(upload(c->d_pg_tdens, c->pg_tdens.data(), c->pg_tdens.size()));
        CK(dalloc(c->d_pg_d, (size_t)std::max(1LL, c->pg_dfloats)));
      }
      c->pg_min = it->second.pg_min;
      c->tune_ms = 0.0;
      return PNFAM_OK;
    }
  }
  cudaStream_t st = c->stream;
  const long long nv = 2 * c->nq * c->nxy;
  CK(cudaMemsetAsync(c->d_state32.p, 0, sizeof(float) * (size_t)nmax * nv, st));
  std::vector<int> list(nmax), flags(P, 0);
  for (int i = 0; i < nmax; ++i) list[i] = i;
  CK(upload(c->d_actlist, list.data(), list.size()));
  const int saved_min = c->pg_min;
  auto t0 = std::chrono::steady_clock::now();
  // device ms of one FP32 evaluation of n points (pair: the pair-tensor path or not)
  auto trial = [&](int n, bool pair, double* ms) -> int {
    for (int i = 0; i < P; ++i) flags[i] = i < n;
    CK(upload(c->d_act32, flags.data(), flags.size()));
    c->pg_min = pair ? 1 : (1 << 30);
    int rc = residual_t<float>(c, P, n, c->d_act32.p, false, st);   // warm
    if (rc) return rc;
    const int reps = 2;
    CK(cudaEventRecord(c->ev[0], st));
    for (int r = 0; r < reps && !rc; ++r) rc = residual_t<float>(c, P, n, c->d_act32.p, false, st);
    if (rc) return rc;
    CK(cudaEventRecord(c->ev[1], st));
    CK(cudaEventSynchronize(c->ev[1]));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, c->ev[0], c->ev[1]));
    *ms = f / reps;
    return PNFAM_OK;
  };
  int rc;
  // 1. density task span (unless PNFAM_GB300_PAIR_KSPAN fixes it)
  if (c->pg_kspan_env <= 0) {
    std::vector<int> cand;
    for (int span : PG_KSPANS) {
      long long tasks = 0;
      for (const PGProb& pr : c->pg_probs)
        if (pr.kind == 1) tasks += (long long)pr.ntile * std::max(1, (pr.nkc + span - 1) / span);
      const double waves = (double)tasks / c->nsm;
      const double last = waves - std::floor(waves);
      if (last == 0.0 || last >= 0.5 || span == PG_KSPANS[0]) cand.push_back(span);
    }
    double best = 1e300;
    int bspan = c->pg_kspan;
    for (int span : cand) {
      pg_density_tasks(c, span);
      CK(upload(c->d_pg_probs, c->pg_probs.data(), c->pg_probs.size()));
      CK(upload(c->d_pg_tdens, c->pg_tdens.data(), c->pg_tdens.size()));
      CK(dalloc(c->d_pg_d, (size_t)std::max(1LL, c->pg_dfloats)));
      double ms = 0.0;
      if ((rc = trial(nmax, true, &ms))) return rc;
      if (ms < best) { best = ms; bspan = span; }
    }
    pg_density_tasks(c, bspan);
    CK(upload(c->d_pg_probs, c->pg_probs.data(), c->pg_probs.size()));
    CK(upload(c->d_pg_tdens, c->pg_tdens.data(), c->pg_tdens.size()));
    CK(dalloc(c->d_pg_d, (size_t)std::max(1LL, c->pg_dfloats)));
  }
  // 2. pair-tensor path from pg_min points on
  if (!c->pg_min_env) {
    std::vector<int> ns;
    std::vector<bool> pair_wins;
    for (int n = 1; n <= nmax; n *= 2) {
      double tp = 0.0, tb = 0.0;
      if ((rc = trial(n, true, &tp)) || (rc = trial(n, false, &tb))) return rc;
      ns.push_back(n);
      pair_wins.push_back(tp <= tb);
    }
    int m = 1 << 30;
    for (int i = (int)ns.size() - 1; i >= 0 && pair_wins[i]; --i) m = ns[i];
    c->pg_min = m;
  } else {
    c->pg_min = saved_min;
  }
  CK(cudaStreamSynchronize(st));
  c->tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = TuneChoice{c->pg_kspan, c->pg_min};
  return PNFAM_OK;
}

// FP32 copies of the ground state and FP32 scratch for P points
static int ensure_buffers32(pnfam_ctx* c, int P) {
  const long long nxy = c->nxy;
  const size_t mo = (size_t)(c->uoff.back() + (long long)c->db.back() * c->db.back());
  if (!c->have32) {
    CK(dalloc(c->d_up32, mo)); CK(dalloc(c->d_vp32, mo)); CK(dalloc(c->d_un32, mo)); CK(dalloc(c->d_vn32, mo));
    CK(dalloc(c->d_phi32, (size_t)5 * c->dqp * c->nghl));
    const double* src[5] = {c->d_up.p, c->d_vp.p, c->d_un.p, c->d_vn.p, c->d_phi.p};
    float* dst[5] = {c->d_up32.p, c->d_vp32.p, c->d_un32.p, c->d_vn32.p, c->d_phi32.p};
    const long long n[5] = {(long long)mo, (long long)mo, (long long)mo, (long long)mo, 5LL * c->dqp * c->nghl};
    for (int k = 0; k < 5; ++k) {
      k_to_f32<<<1024, 256, 0, c->stream>>>(src[k], dst[k], n[k], 1, 0, nullptr);
      CK(cudaGetLastError());
    }
    c->have32 = true;
  }
  // QP-state arrays: nv = Re and Im of X, Y (and P, Q in the statistical FAM); GEMM
  // scratch as in the FP64 form
  const long long nv = 2 * c->nq * nxy;
  const long long tpl = std::max(c->tplane, 8 * nxy);
  CK(dalloc(c->d_state32, (size_t)P * nv));
  CK(dalloc(c->d_T32, (size_t)P * 2 * tpl));
  CK(dalloc(c->d_rsp32, (size_t)P * 8 * nxy));
  CK(dalloc(c->d_hsp32, (size_t)P * 8 * nxy));
  CK(dalloc(c->d_hqp32, (size_t)P * nv));
  CK(dalloc(c->d_dpart32, (size_t)P * 2 * c->G * 2 * ND * c->nghl));
  CK(dalloc(c->d_mf32, (size_t)P * 2 * NMF * 2 * c->nghl));
  CK(dalloc(c->d_xsave, (size_t)P * nv));
  CK(dalloc(c->d_radd, (size_t)P * nv));
  CK(dalloc(c->d_dmax, (size_t)P));
  CK(dalloc(c->d_lastf, (size_t)P * nv));
  CK(dalloc(c->d_lastv, (size_t)P * nv));
  CK(dalloc(c->d_tf, (size_t)P * nv));
  CK(dalloc(c->d_tv, (size_t)P * nv));
  if (c->tc_density) {
    CK(dalloc(c->d_bsplit, (size_t)P * c->bstride));
    if (!c->have_aphi) {
      const int ntr = (c->nghl + 31) / 32, na = (int)c->achunks.size();
      CK(dalloc(c->d_aphi, (size_t)ntr * na * DTC2_ACH));
      if (na > 0) {
        k_dens_asplit<<<dim3(na, ntr), 256, 0, c->stream>>>(c->devbasis<float>(), c->d_achunks.p, na, c->d_aphi.p);
        CK(cudaGetLastError());
      }
      c->have_aphi = true;
    }
  }
  BufDescT<float> bd[NBUF];
  bd[B_UP] = {c->d_up32.p, 0, 0};
  bd[B_VP] = {c->d_vp32.p, 0, 0};
  bd[B_UN] = {c->d_un32.p, 0, 0};
  bd[B_VN] = {c->d_vn32.p, 0, 0};
  bd[B_STATE] = {c->d_state32.p, nv, nv / 2};
  bd[B_T] = {c->d_T32.p, 2 * tpl, tpl};
  bd[B_RSP] = {c->d_rsp32.p, 8 * nxy, 4 * nxy};
  bd[B_HSP] = {c->d_hsp32.p, 8 * nxy, 4 * nxy};
  bd[B_HQP] = {c->d_hqp32.p, nv, nv / 2};
  CK(upload(c->d_bufs32, bd, NBUF));
  if (!c->have_hphi) {
    const int nrc = (c->nghl + HTC_K - 1) / HTC_K;
    CK(dalloc(c->d_hphi, (size_t)std::max(1LL, c->hphi_floats)));
    if (!c->hptiles.empty()) {
      k_hproj_bsplit<<<dim3((unsigned)c->hptiles.size(), 5 * nrc), 256, 0, c->stream>>>(
          c->devbasis<float>(), c->d_hptiles.p, nrc, c->d_hphi.p);
      CK(cudaGetLastError());
    }
    c->have_hphi = true;
  }
  if (!c->have_gsplit) {
    CK(dalloc(c->d_gsplit, (size_t)std::max(1LL, c->gsplit_floats)));
    TaskListTC* lists[4] = {&c->t1a, &c->t1b, &c->t2a, &c->t2b};
    for (TaskListTC* tl : lists) {
      int mc = 0;
      for (const GemmTaskTC& t : tl->tasks) mc = std::max(mc, t.nterm * ((t.K + GTC_K - 1) / GTC_K));
      if (tl->tasks.empty() || mc == 0) continue;
      k_gemm_bsplit<<<dim3((unsigned)tl->tasks.size(), (unsigned)mc), 256, 0, c->stream>>>(tl->d_tasks.p,
                                                                                      c->d_bufs32.p, c->d_gsplit.p);
      CK(cudaGetLastError());
    }
    c->have_gsplit = true;
  }
  {
    const int rc = pg_build(c);
    if (rc) return rc;
  }
  return pg_autotune(c, P);
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
// host half of the basis set-up: block sizes, starts, TR partners, U/V offsets
static int host_basis(pnfam_ctx* c, int nb, int nghl, const int* db, const int* nup) {
  if (nb <= 0 || nb % 2 || nghl <= 0) return fail(PNFAM_EINVAL, "pnfam_gpu_init: nb must be positive and even, nghl positive");
  c->nb = nb;
  c->nghl = nghl;
  c->db.assign(db, db + nb);
  c->maxdb = *std::max_element(c->db.begin(), c->db.end());
  c->nup.assign(nup, nup + nb);
  c->st.resize(nb);
  c->tr.resize(nb);
  c->uoff.resize(nb);
  long long mo = 0;
  int s = 0;
  for (int i = 0; i < nb; ++i) {
    if (c->db[i] < 0 || c->nup[i] < 0 || c->nup[i] > c->db[i])
      return fail(PNFAM_EINVAL, "pnfam_gpu_init: bad block size or spin count");
    c->st[i] = s; s += c->db[i];
    c->uoff[i] = mo; mo += (long long)c->db[i] * c->db[i];
    c->tr[i] = i < nb / 2 ? i + nb / 2 : i - nb / 2;
  }
  for (int i = 0; i < nb; ++i)
    if (c->db[i] != c->db[c->tr[i]]) return fail(PNFAM_EINVAL, "pnfam_gpu_init: TR partner blocks differ in size");
  c->dqp = s;
  return PNFAM_OK;
}

extern "C" int pnfam_gpu_init(const pnfam_basis_t* basis, const double* Ep, const double* En,
                              const double* Up, const double* Vp, const double* Un, const double* Vn,
                              const double* phi, const double* wdcori, const pnfam_coupl_t* coupl,
                              pnfam_ctx_t** out) {
  g_err.clear();
  if (!basis || !Ep || !En || !Up || !Vp || !Un || !Vn || !phi || !wdcori || !coupl || !out)
    return fail(PNFAM_EINVAL, "pnfam_gpu_init: NULL argument");
  *out = nullptr;
  if (basis->nb <= 0 || basis->nb % 2 || basis->nghl <= 0)
    return fail(PNFAM_EINVAL, "pnfam_gpu_init: nb must be positive and even, nghl positive");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(PNFAM_ECUDA, "pnfam_gpu_init: no CUDA device available");
  pnfam_ctx* c = new pnfam_ctx();
  cudaGetDevice(&c->dev);
  {
    const int rcb = host_basis(c, basis->nb, basis->nghl, basis->db, basis->num_spin_up);
    if (rcb) { delete c; return rcb; }
  }
  {
    // FP32 densities on the tensor cores unless PNFAM_GB300_TC_DENSITY=0 (SIMT kernel)
    const char* v = std::getenv("PNFAM_GB300_TC_DENSITY");
    c->tc_density = !(v && v[0] == '0');
    v = std::getenv("PNFAM_GB300_PAIR_GEMM");
    c->pg_mode = (v && v[0] == '0') ? 0 : 1;
    v = std::getenv("PNFAM_GB300_PAIR_GEMM_GB");
    if (v && std::atof(v) > 0) c->pg_budget = std::atof(v) * 1e9;
    v = std::getenv("PNFAM_GB300_PAIR_MIN");
    if (v && std::atoi(v) > 0) { c->pg_min = std::atoi(v); c->pg_min_env = true; }
    v = std::getenv("PNFAM_GB300_AUTOTUNE");
    c->autotune = !(v && v[0] == '0');
    v = std::getenv("PNFAM_GB300_PAIR_KSPAN");
    if (v && std::atoi(v) > 0) c->pg_kspan_env = std::atoi(v);
    v = std::getenv("PNFAM_GB300_PAIR_SMEM_KB");
    if (v && std::atoi(v) >= 64) c->pg_smem = std::min(std::atoi(v), PG_SMEM_MAX / 1024) * 1024;
  }
  const int s = c->dqp;
  const long long mo = c->uoff.back() + (long long)c->db.back() * c->db.back();
  c->ns.resize(s);
  for (int k = 0; k < s; ++k) {
    if (basis->ns[k] != 1 && basis->ns[k] != -1) { delete c; return fail(PNFAM_EINVAL, "pnfam_gpu_init: ns must be +-1"); }
    c->ns[k] = (signed char)basis->ns[k];
  }
  for (int i = 0; i < 12; ++i) c->sc[i] = coupl->scalars[i];
  auto up = [&](auto& buf, const auto* h, size_t n) -> int { CK(upload(buf, h, n)); return 0; };
  int rc = 0;
  const size_t nphi = (size_t)5 * s * c->nghl;
  if ((rc = up(c->d_db, c->db.data(), c->nb)) || (rc = up(c->d_st, c->st.data(), c->nb)) ||
      (rc = up(c->d_nup, c->nup.data(), c->nb)) || (rc = up(c->d_ns, c->ns.data(), (size_t)s)) ||
      (rc = up(c->d_up, Up, (size_t)mo)) || (rc = up(c->d_vp, Vp, (size_t)mo)) ||
      (rc = up(c->d_un, Un, (size_t)mo)) || (rc = up(c->d_vn, Vn, (size_t)mo)) ||
      (rc = up(c->d_ep, Ep, (size_t)s)) || (rc = up(c->d_en, En, (size_t)s)) ||
      (rc = up(c->d_phi, phi, nphi)) || (rc = up(c->d_wd, wdcori, (size_t)c->nghl)) ||
      (rc = up(c->d_crho, coupl->crho, (size_t)c->nghl)) || (rc = up(c->d_cs, coupl->cs, (size_t)c->nghl)) ||
      (rc = up(c->d_cpair, coupl->cpair, (size_t)c->nghl)) || (rc = up(c->d_cspair, coupl->cspair, (size_t)c->nghl))) {
    delete c;
    return rc;
  }
  // the context's main stream (FP32 increment evaluations, Broyden) at the highest
  // priority, the FP64 anchor stream at the lowest: the block scheduler then gives SMs
  // to the tensor-core and bandwidth-bound kernels first and fills what they leave (an
  // SM running one pair-GEMM CTA keeps 100 KB of shared memory and most registers free)
  // with CTAs of the FP64-pipe-bound anchor kernels
  // (PNFAM_GB300_ANCHOR_PRIORITY=high swaps the two)
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  {
    const char* v = std::getenv("PNFAM_GB300_ANCHOR_PRIORITY");
    if (v && std::string(v) == "high") std::swap(prio_lo, prio_hi);
  }
  if (cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
      cudaEventCreate(&c->ev[0]) != cudaSuccess || cudaEventCreate(&c->ev[1]) != cudaSuccess ||
      cudaEventCreate(&c->evt[0]) != cudaSuccess || cudaEventCreate(&c->evt[1]) != cudaSuccess ||
      cudaStreamCreateWithPriority(&c->stream64, cudaStreamNonBlocking, prio_lo) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->evf[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->evf[1], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->evd, cudaEventDisableTiming) != cudaSuccess) {
    delete c;
    return fail(PNFAM_ECUDA, "pnfam_gpu_init: stream/event creation failed");
  }
  if (cudaFuncSetAttribute(k_hproj_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)hproj_fp64_smem_bytes()) != cudaSuccess ||
      cudaFuncSetAttribute(k_hproj_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)hproj_tc_smem_bytes(HTC_MAXN)) != cudaSuccess ||
      cudaFuncSetAttribute(k_density_tc2, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)density_tc2_smem_bytes()) != cudaSuccess ||
      cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)gemm_tc_smem_bytes()) != cudaSuccess ||
      cudaFuncSetAttribute(k_pg_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, PG_SMEM_MAX) != cudaSuccess) {
    delete c;
    return fail(PNFAM_ECUDA, "pnfam_gpu_init: cannot configure shared memory");
  }
  *out = c;
  return PNFAM_OK;
}

// block structures of the QP quadrants from F's block map (host): X = U1^T F V2
// (row i -> tr fc i), Y = V1^T F U2 (i -> fc tr i) and, statistical, P = U1^T F U2
// (i -> fc i), Q = V1^T F V2 (i -> tr fc tr i); all hold nxy elements
static int host_structure(pnfam_ctx* c, int beta_minus, const int* fcols) {
  const int nb = c->nb;
  c->beta_minus = beta_minus ? 1 : 0;
  c->fc.assign(fcols, fcols + nb);
  for (int i = 0; i < nb; ++i)
    if (c->fc[i] < -1 || c->fc[i] >= nb) return fail(PNFAM_EINVAL, "pnfam_gpu_set_operator: fcols out of range");
  c->xc.assign(nb, -1); c->yc.assign(nb, -1); c->xtc.assign(nb, -1); c->ytc.assign(nb, -1);
  c->pc.assign(nb, -1); c->qc.assign(nb, -1);
  for (int i = 0; i < nb; ++i) {
    if (c->fc[i] >= 0) c->xc[i] = c->tr[c->fc[i]];
    c->yc[i] = c->fc[c->tr[i]];
    c->pc[i] = c->fc[i];
    if (c->yc[i] >= 0) c->qc[i] = c->tr[c->yc[i]];
  }
  for (int i = 0; i < nb; ++i) {
    if (c->xc[i] >= 0) { if (c->xtc[c->xc[i]] >= 0) return fail(PNFAM_EINVAL, "pnfam_gpu_set_operator: F is not one block per column"); c->xtc[c->xc[i]] = i; }
    if (c->yc[i] >= 0) { if (c->ytc[c->yc[i]] >= 0) return fail(PNFAM_EINVAL, "pnfam_gpu_set_operator: F is not one block per column"); c->ytc[c->yc[i]] = i; }
  }
  long long nf, nx, ny, nxt, nyt, np_, nq_;
  c->foff = offsets(c->fc, c->db, &nf);
  c->xoff = offsets(c->xc, c->db, &nx);
  c->yoff = offsets(c->yc, c->db, &ny);
  c->xtoff = offsets(c->xtc, c->db, &nxt);
  c->ytoff = offsets(c->ytc, c->db, &nyt);
  c->poff = offsets(c->pc, c->db, &np_);
  c->qoff = offsets(c->qc, c->db, &nq_);
  if (nf != nx || nf != ny || nf != nxt || nf != nyt || nf != np_ || nf != nq_ || nf == 0)
    return fail(PNFAM_EINVAL, "pnfam_gpu_set_operator: inconsistent block structure");
  // the statistical quadrants keep the symmetry fc[tr fc[i]] = tr i that their tasks use
  if (c->nq == 4)
    for (int i = 0; i < nb; ++i)
      if (c->fc[i] >= 0 && c->fc[c->tr[c->fc[i]]] != c->tr[i])
        return fail(PNFAM_EINVAL, "pnfam_gpu_set_operator: F block map is not symmetric under time reversal");
  c->nxy = nf;
  return PNFAM_OK;
}

extern "C" int pnfam_gpu_set_operator(pnfam_ctx_t* c, int beta_minus, const int* fcols, const double* Fsp,
                                      int n_xterms, const double* const* Gsp) {
  g_err.clear();
  if (!c || !fcols || !Fsp || n_xterms < 0 || (n_xterms > 0 && !Gsp))
    return fail(PNFAM_EINVAL, "pnfam_gpu_set_operator: bad argument");
  const int nb = c->nb;
  {
    const int rcs = host_structure(c, beta_minus, fcols);
    if (rcs) return rcs;
  }
  const long long nf = c->nxy;
  c->nops = 1 + n_xterms;
  CK(upload(c->d_fc, c->fc.data(), nb));
  CK(upload(c->d_xtc, c->xtc.data(), nb));
  CK(upload(c->d_ytc, c->ytc.data(), nb));
  CK(upload(c->d_foff, c->foff.data(), nb));
  CK(upload(c->d_xtoff, c->xtoff.data(), nb));
  CK(upload(c->d_ytoff, c->ytoff.data(), nb));
  // element -> (row state, column state) for the X|Y[|P|Q] layout (Green's function)
  const int nq = c->nq;
  std::vector<int> erow(nq * nf), ecol(nq * nf);
  for (int part = 0; part < nq; ++part) {
    const std::vector<int>& cols = part == 0 ? c->xc : part == 1 ? c->yc : part == 2 ? c->pc : c->qc;
    const std::vector<long long>& off = part == 0 ? c->xoff : part == 1 ? c->yoff : part == 2 ? c->poff : c->qoff;
    for (int i = 0; i < nb; ++i) {
      if (cols[i] < 0) continue;
      const int d = c->db[i], dc = c->db[cols[i]];
      for (int b = 0; b < dc; ++b)
        for (int a = 0; a < d; ++a) {
          const long long e = part * nf + off[i] + a + (long long)b * d;
          erow[e] = c->st[i] + a;
          ecol[e] = c->st[cols[i]] + b;
        }
    }
  }
  CK(upload(c->d_erow, erow.data(), erow.size()));
  CK(upload(c->d_ecol, ecol.data(), ecol.size()));
  // partition of the density work
  {
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->dev);
    c->nsm = std::max(nsm, 1);
    const int ntr = (c->nghl + DRT - 1) / DRT;
    int nrows = 0;
    for (int i = 0; i < nb; ++i) nrows += c->fc[i] >= 0;
    c->G = std::max(1, std::min(nrows, (2 * std::max(nsm, 1) + ntr - 1) / ntr));
  }
  c->nchunk_bro = (int)((2 * nq * nf + BRO_CHUNK - 1) / BRO_CHUNK);
  c->nchunk_c = (int)std::min<long long>(32, std::max<long long>(1, (nq * nf) / 4096));
  build_tasks(c);
  pg_setup(c);
  CK(c->k1a.finalize()); CK(c->k1b.finalize()); CK(c->k2a.finalize()); CK(c->k2b.finalize());
  {
    TaskList* src[4] = {&c->k1a, &c->k1b, &c->k2a, &c->k2b};
    TaskListTC* dst[4] = {&c->t1a, &c->t1b, &c->t2a, &c->t2b};
    long long goff = 0;
    for (int k = 0; k < 4; ++k) {
      dst[k]->build(*src[k]);
      for (GemmTaskTC& t : dst[k]->tasks) {
        if (t.ncols > 256) return fail(PNFAM_EINVAL, "pnfam_gpu_set_operator: block larger than 256");
        t.bsoff = goff;   // the task's pre-split ground-state chunks
        goff += (long long)t.nterm * ((t.K + GTC_K - 1) / GTC_K) * t.npad * 2 * GTC_K;
      }
      CK(upload(dst[k]->d_tasks, dst[k]->tasks.data(), dst[k]->tasks.size()));
    }
    c->gsplit_floats = goff;
    c->have_gsplit = false;
  }
  CK(upload(c->d_htasks, c->htasks.data(), c->htasks.size()));
  CK(upload(c->d_htasks_tc, c->htasks_tc.data(), c->htasks_tc.size()));
  CK(upload(c->d_hptiles, c->hptiles.data(), c->hptiles.size()));
  CK(upload(c->d_dunits0, c->dunits[0].data(), c->dunits[0].size()));
  CK(upload(c->d_dunits1, c->dunits[1].data(), c->dunits[1].size()));
  CK(upload(c->d_bchunks, c->bchunks.data(), c->bchunks.size()));
  if (!c->have_aphi) CK(upload(c->d_achunks, c->achunks.data(), c->achunks.size()));
  c->have_op = true;
  int rc = ensure_buffers(c, std::max(1, c->cap_P), std::max(1, c->cap_M));
  if (rc) return rc;
  c->cap_P = std::max(1, c->cap_P); c->cap_M = std::max(1, c->cap_M);
  // F_qp and cross terms: K2 applied to dH_sp = (F, 0, 0, 0) (pnfam_solver.f90:368-381)
  CK(dalloc(c->d_fops, (size_t)c->nops * nq * nf));
  std::vector<int> one = {1};
  CK(upload(c->d_active, one.data(), 1));
  for (int k = 0; k < c->nops; ++k) {
    const double* src = k == 0 ? Fsp : Gsp[k - 1];
    CK(cudaMemsetAsync(c->d_hsp.p, 0, sizeof(double) * 8 * nf, c->stream));
    CK(cudaMemcpyAsync(c->d_hsp.p, src, sizeof(double) * nf, cudaMemcpyHostToDevice, c->stream));
    if ((rc = launch_gemm(c, c->k2a, 1, c->d_active.p))) return rc;
    if ((rc = launch_gemm(c, c->k2b, 1, c->d_active.p))) return rc;
    CK(cudaMemcpyAsync(c->d_fops.p + (long long)k * nq * nf, c->d_hqp.p, sizeof(double) * nq * nf,
                       cudaMemcpyDeviceToDevice, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return PNFAM_OK;
}

// ---------------------------------------------------------------------------
// Solve engine: P slots on one context, each slot one omega point with its own
// iteration counter and Broyden history (pnfam_solver.f90:114-209 per slot).
// A slot is admitted with a point, iterated one evaluation per launch/finish
// pair, and retired when it converges or reaches max_iter; a retired slot can
// take the next point while the others keep iterating (continuous batching).
// ---------------------------------------------------------------------------
struct pnfam_engine {
  pnfam_ctx* c = nullptr;
  pnfam_solver_opts_t o{};
  int P = 0, M = 0, bmode = BRO_BROYDEN, N = 0, nops = 1;
  long long nxy = 0;
  bool no_res = false, mixed = false, timed = false;
  double switch_si = 0.0;
  // opts.reserved[3] > 0: convergence also asks every strength value to have settled,
  // |S - S_prev| <= s_rel |S| + 1e-13 max|S| on Re and Im of each value (at most
  // EXTRA iterations beyond si < epsilon)
  double s_rel = 0.0;
  static constexpr int EXTRA = 20;
  // "near" its anchor: max|X - X_a| <= near * epsilon (opts.reserved[4] = n > 0: 10^n;
  // default 1000), where the FP32 error of an increment evaluation is far below epsilon
  double near = 1000.0;
  // a stall of the increment iteration counts as the FP32 noise floor (and takes an
  // anchor) only while si <= FLOOR * max|d|: far above that, FP32 rounding of the
  // increment cannot be what holds the residual up, and an anchor would not help
  static constexpr double FLOOR = 1e-3;
  // per slot (host)
  std::vector<int> active, it, anchor, since_best, nstall, fresh;
  std::vector<long long> tag;
  std::vector<double> si, sre, sim, best, wre, wim, pre, pim;
  std::vector<int> extra;
  // restart: slots admitted with a stored state vector (their first iteration evaluates
  // the field of that state instead of starting from X = 0) and the vectors still to be
  // copied in at the next launch
  std::vector<int> x0;
  std::vector<std::pair<int, std::vector<double>>> x0q;
  std::vector<unsigned long long> hdmax;
  std::vector<int> pint, act32, act64, actlist;
  // Asynchronous anchors (mixed form): when a launch has FP32 increment evaluations,
  // the FP64 anchor evaluations it also needs run as a batch on the context's second
  // stream and their slots are parked (afly 1) while the engine keeps stepping its
  // other slots; a later launch finds the batch complete (its event), and each parked
  // slot then takes the Green's function and Broyden step of that anchor (afly 2, then
  // 0).  A slot's arithmetic is the same as with the anchor inside one launch; only
  // the anchor's FP64 work no longer holds up the other slots.  stepped: the slots
  // that step in the launch in flight.
  bool async = false;   // opts.reserved[5]
  std::vector<int> afly, stepped;
  struct ABatch { int ring; std::vector<int> slots; };
  std::deque<ABatch> abatch;
  cudaEvent_t aev[ANCH_RING] = {};
  int aring = 0;
  PinBuf<int> pin_a;   // [ANCH_RING][P] the batches' slot flags
  ~pnfam_engine() {
    for (cudaEvent_t& ev : aev)
      if (ev) cudaEventDestroy(ev);
  }
  int herr = 0;
  std::vector<double> hsi, cpart;
  // pinned staging of the per-evaluation copies: ints [active P | pint 6P | act64 P |
  // act32 P | actlist P | err 1], doubles [wre P | wim P | si P | cpart], dmax [P]
  PinBuf<int> pin_i;
  PinBuf<double> pin_d;
  PinBuf<unsigned long long> pin_u;
  double* hist = nullptr;   // optional [P][max_iter+1][3] (batch solve only)
  bool dirty_w = true;
  int pending = 0;          // an evaluation is in flight
  struct Done { long long tag; int slot, iters; double si; };
  std::vector<Done> done;
  std::vector<double> done_re, done_im;  // [ndone][nops]
};

// a context freed before its engine leaves the engine without a context
void pnfam_ctx::detach_engine() {
  if (engine) {
    cudaStreamSynchronize(stream64);
    cudaStreamSynchronize(stream);
    engine->c = nullptr;
    engine->pending = 0;
    engine = nullptr;
  }
}

static int engine_setup(pnfam_engine* e, pnfam_ctx* c, int P, const pnfam_solver_opts_t* o) {
  if (!c->have_op) return fail(PNFAM_ESTATE, "call pnfam_gpu_set_operator first");
  if (o->max_iter < 0) return fail(PNFAM_EINVAL, "max_iter < 0");
  if (o->precision != 0 && o->precision != 1)
    return fail(PNFAM_EINVAL, "precision must be 0 (FP64) or 1 (mixed FP32/FP64)");
  e->c = c; e->o = *o; e->P = P;
  e->no_res = std::fabs(o->quench_residual_int) < 1e-10;
  e->M = e->no_res ? -1 : o->broyden_history_size;
  if (e->M > 64) return fail(PNFAM_EINVAL, "broyden_history_size > 64 is not supported");
  e->bmode = e->M < 0 ? BRO_NOMIX : e->M == 0 ? BRO_LINEAR : BRO_BROYDEN;
  e->nxy = c->nxy; e->N = (int)(2 * c->nq * c->nxy); e->nops = c->nops;
  int rc = ensure_buffers(c, std::max(P, c->cap_P), std::max(std::max(e->M, 1), c->cap_M));
  if (rc) return rc;
  c->cap_P = std::max(P, c->cap_P); c->cap_M = std::max(std::max(e->M, 1), c->cap_M);
  e->mixed = o->precision == 1 && !e->no_res;
  if (e->mixed && (rc = ensure_buffers32(c, c->cap_P))) return rc;
  // Mixed form (precision 1): one Broyden iteration per evaluation, as in the FP64
  // form, but the residual interaction is evaluated in FP32 on the increment
  // d = X - X_a from an anchor X_a whose image g(X_a) is known in FP64:
  //   g(X) = g(X_a) + G o (q H(d))    (H is linear; increment evaluation, FP32)
  // The FP32 error of an increment evaluation scales with |d|, not |X|.  An anchor
  // evaluation computes g(X) entirely in FP64 and makes X the new anchor.
  // Iteration 0 is the anchor X_a = 0, g(0) = G o F, exact without a field
  // evaluation.  A point is "near" its anchor while max|d| <= NEAR*epsilon, where
  // the FP32 error is far below epsilon.  Convergence (si < epsilon) is accepted on
  // an anchor or on a near increment evaluation; a far point takes an FP64 anchor
  // when si < 10^-reserved[1] (default 100*epsilon) or si stops falling at the FP32
  // noise floor (si <= FLOOR*max|d|).  Every evaluation counts against max_iter.
  e->switch_si = o->reserved[1] > 0 ? std::pow(10.0, -o->reserved[1]) : 100.0 * o->convergence_epsilon;
  e->timed = o->reserved[0] != 0;
  e->s_rel = o->reserved[3] > 0 ? std::pow(10.0, -o->reserved[3]) : 0.0;
  e->near = o->reserved[4] > 0 ? std::pow(10.0, o->reserved[4]) : 1000.0;
  e->async = o->reserved[5] != 0;
  c->live = o->reserved[2] != 0;
  c->nlev = 0;
  c->live_ms[0] = c->live_ms[1] = 0.0;
  c->live_n[0] = c->live_n[1] = 0;
  const int nops = e->nops;
  e->active.assign(P, 0); e->it.assign(P, 0); e->anchor.assign(P, 1); e->since_best.assign(P, 0);
  e->nstall.assign(P, 0); e->fresh.assign(P, 0); e->tag.assign(P, -1);
  e->si.assign(P, 1.0); e->sre.assign((size_t)P * nops, 0.0); e->sim.assign((size_t)P * nops, 0.0);
  e->pre.assign((size_t)P * nops, 0.0); e->pim.assign((size_t)P * nops, 0.0); e->extra.assign(P, 0);
  e->x0.assign(P, 0); e->x0q.clear();
  e->best.assign(P, 1e300); e->wre.assign(P, 0.0); e->wim.assign(P, 0.0); e->hdmax.assign(P, 0);
  e->pint.assign((size_t)6 * P, 0); e->act32.assign(P, 0); e->act64.assign(P, 0);
  e->afly.assign(P, 0); e->stepped.assign(P, 0); e->abatch.clear(); e->aring = 0;
  for (cudaEvent_t& ev : e->aev)
    if (!ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  CK(e->pin_a.ensure((size_t)ANCH_RING * P));
  e->hsi.assign(P, 0.0); e->cpart.assign((size_t)P * c->nchunk_c * 2 * nops, 0.0);
  CK(e->pin_i.ensure((size_t)10 * P + 1));
  CK(e->pin_d.ensure((size_t)3 * P + e->cpart.size()));
  CK(e->pin_u.ensure((size_t)P));
  for (int k = 0; k < 8; ++k) c->stage_ms[k] = 0.0;
  for (int k = 0; k < 5; ++k) c->stage32_ms[k] = 0.0;
  c->pit64 = 0; c->pit32 = 0; c->launches = 0;
  return PNFAM_OK;
}

static void engine_retire(pnfam_engine* e, int p, int iters) {
  e->done.push_back({e->tag[p], p, iters, e->si[p]});
  for (int k = 0; k < e->nops; ++k) {
    e->done_re.push_back(e->sre[(size_t)p * e->nops + k]);
    e->done_im.push_back(e->sim[(size_t)p * e->nops + k]);
  }
  e->active[p] = 0;
}

static void engine_hist(pnfam_engine* e, int p) {
  if (!e->hist) return;
  double* h = e->hist + ((size_t)p * (e->o.max_iter + 1) + e->it[p]) * 3;
  h[0] = e->si[p]; h[1] = e->sre[(size_t)p * e->nops]; h[2] = e->sim[(size_t)p * e->nops];
}

// admit up to n points into free slots; returns the number admitted
static int engine_admit(pnfam_engine* e, int n, const double* re_w, const double* im_w, const long long* tags) {
  int k = 0;
  for (int p = 0; p < e->P && k < n; ++p) {
    if (e->active[p]) continue;
    e->active[p] = 1; e->it[p] = 0; e->anchor[p] = 1; e->since_best[p] = 0; e->nstall[p] = 0;
    e->best[p] = 1e300; e->si[p] = 1.0; e->fresh[p] = 1; e->extra[p] = 0; e->x0[p] = 0; e->afly[p] = 0;
    for (int q = 0; q < e->nops; ++q) { e->sre[(size_t)p * e->nops + q] = 0.0; e->sim[(size_t)p * e->nops + q] = 0.0; }
    e->wre[p] = re_w[k]; e->wim[p] = im_w[k];
    e->tag[p] = tags ? tags[k] : k;
    e->dirty_w = true;
    engine_hist(e, p);
    if (e->o.max_iter == 0) engine_retire(e, p, -1);
    ++k;
  }
  return k;
}

// The reference's Broyden vector (pnfam_broyden.f90:47-60) orders the parts
// Re X, Re Y, Im X, Im Y[, Re P, Re Q, Im P, Im Q]; a slot's device state is
// [Re X|Y[|P|Q] | Im X|Y[|P|Q]].  Both are the same for nq = 2.  Part j (nf doubles)
// of the reference vector sits at part state_part(nq, j) of the device state.
static inline int state_part(int nq, int j) {
  if (nq == 2) return j;
  static const int map4[8] = {0, 1, 4, 5, 2, 3, 6, 7};
  return map4[j];
}
static void state_from_ref(int nq, long long nf, const double* ref, double* dev) {
  for (int j = 0; j < 2 * nq; ++j)
    std::copy(ref + j * nf, ref + (j + 1) * nf, dev + state_part(nq, j) * nf);
}
static void state_to_ref(int nq, long long nf, const double* dev, double* ref) {
  for (int j = 0; j < 2 * nq; ++j)
    std::copy(dev + state_part(nq, j) * nf, dev + (state_part(nq, j) + 1) * nf, ref + j * nf);
}

// restart: slot p (just admitted, not yet launched) starts from the state vector x
// (N doubles in the reference's Broyden order)
static int engine_set_state(pnfam_engine* e, int p, const double* x) {
  if (p < 0 || p >= e->P || !e->active[p] || e->it[p] != 0)
    return fail(PNFAM_ESTATE, "a start vector needs a slot that was just admitted");
  e->x0[p] = 1;
  std::vector<double> v(e->N);
  state_from_ref((int)(e->N / (2 * e->nxy)), e->nxy, x, v.data());
  e->x0q.emplace_back(p, std::move(v));
  return PNFAM_OK;
}

// one Broyden step of every active slot: FP64 history (FP64 form), pair-arithmetic
// history (mixed form)
static int broyden_step(pnfam_ctx* c, pnfam_engine* e, int any_bro, const int* d_itp, const int* d_mode) {
  const int P = e->P, N = e->N;
  const int* act = c->d_active.p;
  BroState S;
  S.N = N; S.M = std::max(e->M, 1); S.alpha = e->o.alpha_mix;
  S.vin = c->d_state.p; S.vout = c->d_vout.p; S.df = c->d_df.p; S.dv = c->d_dv.p;
  S.part = c->d_bpart.p; S.nchunk = c->nchunk_bro;
  S.itp = d_itp; S.modep = d_mode;
  BroState2 S2;
  S2.N = N; S2.M = S.M; S2.alpha = S.alpha; S2.vin = S.vin; S2.vout = S.vout;
  S2.df = reinterpret_cast<float2*>(c->d_df.p); S2.u = reinterpret_cast<float2*>(c->d_dv.p);
  S2.lastf = c->d_lastf.p; S2.lastv = c->d_lastv.p; S2.tf = c->d_tf.p; S2.tv = c->d_tv.p;
  S2.part = S.part; S2.nchunk = S.nchunk; S2.itp = d_itp; S2.modep = d_mode;
  const bool pair = e->mixed;
  const double w0 = 0.01;
  dim3 grid(c->nchunk_bro, P);
  if (pair) k_bro_diff2<<<grid, 256, 0, c->stream>>>(S2, act);
  else k_bro_diff<<<grid, 256, 0, c->stream>>>(S, act);
  k_bro_solve<<<P, 256, 0, c->stream>>>(S, 0, w0, c->d_si.p, c->d_norm.p, c->d_beta.p, c->d_gamma.p, act);
  c->launches += 2;
  if (any_bro) {
    if (pair) k_bro_dots2<<<grid, 256, 0, c->stream>>>(S2, c->d_norm.p, act);
    else k_bro_dots<<<grid, 256, 0, c->stream>>>(S, c->d_norm.p, act);
    k_bro_solve<<<P, 256, 0, c->stream>>>(S, 1, w0, c->d_si.p, c->d_norm.p, c->d_beta.p, c->d_gamma.p, act);
    c->launches += 2;
  }
  dim3 ug((unsigned)std::min<long long>(4096, (N + 255) / 256), P);
  if (pair) k_bro_update2<<<ug, 256, 0, c->stream>>>(S2, c->d_gamma.p, act);
  else k_bro_update<<<ug, 256, 0, c->stream>>>(S, c->d_gamma.p, act);
  c->launches++;
  CK(cudaGetLastError());
  return PNFAM_OK;
}

// enqueue one evaluation (and Broyden step) for every active slot that is not parked
// on an anchor in flight.  block_if_idle: when every active slot is parked, wait for
// the oldest anchor batch instead of returning with nothing launched.
static int engine_launch(pnfam_engine* e, bool block_if_idle) {
  pnfam_ctx* c = e->c;
  const int P = e->P, N = e->N;
  const long long nxy = e->nxy;
  const bool timed = e->timed;
  // anchor batches that have completed: their slots step in this launch
  std::vector<int> resumed_ev;
  auto resume_front = [&]() {
    const pnfam_engine::ABatch& b = e->abatch.front();
    for (int p : b.slots) e->afly[p] = 2;
    resumed_ev.push_back(b.ring);
    e->abatch.pop_front();
  };
  while (!e->abatch.empty()) {
    const cudaError_t q = cudaEventQuery(e->aev[e->abatch.front().ring]);
    if (q == cudaErrorNotReady) break;
    if (q != cudaSuccess) return fail(PNFAM_ECUDA, std::string("anchor batch: ") + cudaGetErrorString(q));
    resume_front();
  }
  {
    int nstep = 0;
    for (int p = 0; p < P; ++p) nstep += e->active[p] && e->afly[p] != 1;
    if (nstep == 0 && !e->abatch.empty()) {
      if (!block_if_idle) return PNFAM_OK;   // nothing can step before an anchor completes
      CK(cudaEventSynchronize(e->aev[e->abatch.front().ring]));
      resume_front();
    }
  }
  // a free ring entry for a new batch
  if ((int)e->abatch.size() == ANCH_RING) {
    CK(cudaEventSynchronize(e->aev[e->abatch.front().ring]));
    resume_front();
  }
  int nact = 0, n32 = 0, n64 = 0, nanch = 0, nfresh = 0, any_bro = 0;
  for (int p = 0; p < P; ++p) {
    const bool a = e->active[p] != 0 && e->afly[p] != 1;   // steps in this launch
    const bool resumed = a && e->afly[p] == 2;            // its anchor was evaluated earlier
    const bool first = a && e->it[p] == 0;
    // the field of X = 0 vanishes: no evaluation at the first iteration, unless the
    // slot starts from a stored state
    const bool zero = first && !e->x0[p];
    const bool lo = e->mixed && !e->anchor[p];
    e->act32[p] = a && lo && !zero;
    e->act64[p] = a && !lo && !zero && !resumed;
    e->stepped[p] = a;
    n32 += e->act32[p]; n64 += e->act64[p];
  }
  // FP64 anchors beside FP32 increments: asynchronous, their slots parked
  const bool async = e->async && e->mixed && !timed && n64 > 0 && n32 > 0;
  std::vector<int> batch;
  if (async)
    for (int p = 0; p < P; ++p)
      if (e->act64[p]) { batch.push_back(p); e->stepped[p] = 0; }
  for (int p = 0; p < P; ++p) {
    const bool a = e->stepped[p] != 0, first = a && e->it[p] == 0;
    if (a && e->afly[p] == 2) e->afly[p] = 0;
    nact += a;
    e->pint[p] = e->it[p];
    e->pint[P + p] = first && e->bmode == BRO_BROYDEN ? BRO_LINEAR : e->bmode;
    e->pint[2 * P + p] = a && e->act32[p];
    e->pint[3 * P + p] = a && e->mixed && e->anchor[p];
    e->pint[4 * P + p] = first && !e->x0[p];
    e->pint[5 * P + p] = a && e->fresh[p];
    nanch += e->pint[3 * P + p]; nfresh += e->pint[5 * P + p];
    any_bro |= a && e->pint[P + p] == BRO_BROYDEN;
    if (a) e->fresh[p] = 0;
  }
  if (nact == 0 && batch.empty()) return PNFAM_OK;
  c->pit32 += n32; c->pit64 += n64;
  // the completed batches (already complete: ordering only) before their slots step
  for (int r : resumed_ev) CK(cudaStreamWaitEvent(c->stream, e->aev[r], 0));
  auto tic = [&]() { if (timed) cudaEventRecord(c->ev[0], c->stream); };
  auto toc = [&](int k) {
    if (!timed) return;
    cudaEventRecord(c->ev[1], c->stream);
    cudaEventSynchronize(c->ev[1]);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
    c->stage_ms[k] += ms;
  };
  int* d_itp = c->d_pint.p;
  int* d_mode = c->d_pint.p + P;
  int* d_incr = c->d_pint.p + 2 * P;
  int* d_anch = c->d_pint.p + 3 * P;
  int* d_zero = c->d_pint.p + 4 * P;
  int* d_fresh = c->d_pint.p + 5 * P;
  const dim3 vgrid((unsigned)std::min<long long>(2048, (N + 255) / 256), P);
  // host-to-device copies through pinned staging (nothing of the previous evaluation
  // is in flight: engine_finish waited for it)
  int* pi_ = e->pin_i.p;
  double* pd_ = e->pin_d.p;
  std::memcpy(pi_, e->stepped.data(), sizeof(int) * P);
  std::memcpy(pi_ + P, e->pint.data(), sizeof(int) * 6 * P);
  CK(cudaMemcpyAsync(c->d_active.p, pi_, sizeof(int) * P, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d_pint.p, pi_ + P, sizeof(int) * 6 * P, cudaMemcpyHostToDevice, c->stream));
  if (e->dirty_w) {
    std::memcpy(pd_, e->wre.data(), sizeof(double) * P);
    std::memcpy(pd_ + P, e->wim.data(), sizeof(double) * P);
    CK(cudaMemcpyAsync(c->d_wre.p, pd_, sizeof(double) * P, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_wim.p, pd_ + P, sizeof(double) * P, cudaMemcpyHostToDevice, c->stream));
    e->dirty_w = false;
  }
  const double* E1 = c->beta_minus ? c->d_ep.p : c->d_en.p;
  const double* E2 = c->beta_minus ? c->d_en.p : c->d_ep.p;
  const int nq = c->nq;
  if (nfresh) {  // newly admitted slots start from X = 0, with their Green's function
    k_vecop<<<vgrid, 256, 0, c->stream>>>(2, 0.0, c->d_state.p, nullptr, N, d_fresh);
    const int gx = (int)std::min<long long>(4096, (nq * nxy + 255) / 256);
    const double* f1 = nq == 4 ? (c->beta_minus ? c->d_fp.p : c->d_fn.p) : nullptr;
    const double* f2 = nq == 4 ? (c->beta_minus ? c->d_fn.p : c->d_fp.p) : nullptr;
    k_green_prep<<<dim3(gx, P), 256, 0, c->stream>>>(nxy, nq, c->d_erow.p, c->d_ecol.p, E1, E2, f1, f2, c->d_wre.p,
                                                     c->d_wim.p, c->d_gfn.p, d_fresh);
    c->launches += 2;
  }
  // stored start vectors (restart) over the zeroed state of their slots
  for (auto& q : e->x0q)
    CK(cudaMemcpyAsync(c->d_state.p + (size_t)q.first * N, q.second.data(), sizeof(double) * N,
                       cudaMemcpyHostToDevice, c->stream));
  e->x0q.clear();
  const int* act = c->d_active.p;
  int rc;
  bool split = false;
  if (!e->no_res) {
    if (async) {
      // FP64 (anchor) evaluations of the parked slots and FP32 increment evaluations of
      // the others use disjoint scratch and write disjoint rows of hqp; the batch runs
      // on the second stream with its own copy of the slot flags
      const int r = e->aring;
      e->aring = (e->aring + 1) % ANCH_RING;
      int* pa = e->pin_a.p + (size_t)r * P;
      int* da = c->d_act64r.p + (size_t)r * P;
      std::memcpy(pa, e->act64.data(), sizeof(int) * P);
      CK(cudaEventRecord(c->evf[0], c->stream));
      CK(cudaStreamWaitEvent(c->stream64, c->evf[0], 0));
      CK(cudaMemcpyAsync(da, pa, sizeof(int) * P, cudaMemcpyHostToDevice, c->stream64));
      if ((rc = residual_t<double>(c, P, n64, da, false, c->stream64))) return rc;
      CK(cudaEventRecord(e->aev[r], c->stream64));
      for (int p : batch) e->afly[p] = 1;
      e->abatch.push_back({r, std::move(batch)});
    } else if (n64) {
      std::memcpy(pi_ + 7 * P, e->act64.data(), sizeof(int) * P);
      CK(cudaMemcpyAsync(c->d_act64.p, pi_ + 7 * P, sizeof(int) * P, cudaMemcpyHostToDevice, c->stream));
      // beside this launch's FP32 increments (disjoint scratch, disjoint rows of hqp):
      // on the second stream, joined before the Green's function (not when timed)
      split = n32 > 0 && !timed;
      if (split) {
        CK(cudaEventRecord(c->evf[0], c->stream));
        CK(cudaStreamWaitEvent(c->stream64, c->evf[0], 0));
      }
      if ((rc = residual_t<double>(c, P, n64, c->d_act64.p, timed, split ? c->stream64 : c->stream))) return rc;
      if (split) CK(cudaEventRecord(c->evf[1], c->stream64));
    }
    if (e->mixed) {
      std::memcpy(pi_ + 8 * P, e->act32.data(), sizeof(int) * P);
      CK(cudaMemcpyAsync(c->d_act32.p, pi_ + 8 * P, sizeof(int) * P, cudaMemcpyHostToDevice, c->stream));
      if (n32) {
        e->actlist.clear();
        for (int p = 0; p < P; ++p)
          if (e->act32[p]) e->actlist.push_back(p);
        std::memcpy(pi_ + 9 * P, e->actlist.data(), sizeof(int) * n32);
        CK(cudaMemcpyAsync(c->d_actlist.p, pi_ + 9 * P, sizeof(int) * n32, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemsetAsync(c->d_dmax.p, 0, sizeof(unsigned long long) * P, c->stream));
        // a few elements per thread and one atomic per block for max|X - X_a|
        const dim3 cgrid((unsigned)std::min<long long>(256, (N + 255) / 256), P);
        k_to_f32<<<cgrid, 256, 0, c->stream>>>(c->d_state.p, c->d_state32.p, N, P, N, c->d_act32.p, c->d_xsave.p,
                                               c->d_dmax.p);
        if ((rc = residual_t<float>(c, P, n32, c->d_act32.p, timed, c->stream))) return rc;
        c->launches++;
        CK(cudaGetLastError());
      }
    }
  }
  if (split) CK(cudaStreamWaitEvent(c->stream, c->evf[1], 0));
  tic();
  {
    const int gx = (int)std::min<long long>(4096, (nq * nxy + 255) / 256);
    k_green<<<dim3(gx, P), 256, 0, c->stream>>>(nxy, nq, P, e->no_res ? nullptr : c->d_hqp.p,
                                                e->mixed ? c->d_hqp32.p : nullptr, c->d_fops.p, c->d_gfn.p,
                                                e->o.quench_residual_int, c->d_vout.p, act,
                                                e->mixed ? d_incr : nullptr, c->d_radd.p, d_zero);
    c->launches++;
    if (nanch) {  // new anchors: X_a = X, g(X_a) = vout
      k_vecop<<<vgrid, 256, 0, c->stream>>>(0, 0.0, c->d_xsave.p, c->d_state.p, N, d_anch);
      k_vecop<<<vgrid, 256, 0, c->stream>>>(0, 0.0, c->d_radd.p, c->d_vout.p, N, d_anch);
      c->launches += 2;
    }
    CK(cudaGetLastError());
  }
  toc(5);
  // ---- Broyden (pnfam_broyden.f90:117-216), each slot at its own iteration ----
  tic();
  if ((rc = broyden_step(c, e, any_bro, d_itp, d_mode))) return rc;
  toc(6);
  tic();
  {
    dim3 grid(c->nchunk_c, P);
    k_contract<<<grid, 256, 0, c->stream>>>(nxy, nq, e->nops, c->d_fops.p, c->d_state.p, c->nchunk_c, c->d_cpart.p,
                                            act);
    c->launches++;
    CK(cudaGetLastError());
  }
  // device-to-host copies into pinned staging: the call returns at once and
  // engine_finish picks the values up after its wait
  CK(cudaMemcpyAsync(pd_ + 2 * P, c->d_si.p, sizeof(double) * P, cudaMemcpyDeviceToHost, c->stream));
  if (e->mixed)
    CK(cudaMemcpyAsync(e->pin_u.p, c->d_dmax.p, sizeof(unsigned long long) * P, cudaMemcpyDeviceToHost,
                       c->stream));
  CK(cudaMemcpyAsync(pd_ + 3 * P, c->d_cpart.p, sizeof(double) * e->cpart.size(), cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaMemcpyAsync(pi_ + 10 * P, c->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaEventRecord(c->evd, c->stream));
  if (timed) toc(7);
  e->pending = 1;
  return PNFAM_OK;
}

// wait for the evaluation in flight, update every active slot and retire the
// slots that converged or reached max_iter
static int engine_finish(pnfam_engine* e) {
  if (!e->pending) return PNFAM_OK;
  pnfam_ctx* c = e->c;
  CK(cudaStreamSynchronize(c->stream));
  e->pending = 0;
  live_collect(c);
  {
    const int P = e->P;
    std::memcpy(e->hsi.data(), e->pin_d.p + 2 * P, sizeof(double) * P);
    std::memcpy(e->cpart.data(), e->pin_d.p + 3 * P, sizeof(double) * e->cpart.size());
    if (e->mixed) std::memcpy(e->hdmax.data(), e->pin_u.p, sizeof(unsigned long long) * P);
    e->herr = e->pin_i.p[10 * P];
  }
  if (e->herr) {
    cudaMemsetAsync(c->d_err.p, 0, sizeof(int), c->stream);
    e->herr = 0;
    return fail(PNFAM_ECUDA, "a wait on the tensor cores gave up (field projection)");
  }
  const pnfam_solver_opts_t& o = e->o;
  const int nops = e->nops;
  const double pi = 3.141592653589793238462643;
  for (int p = 0; p < e->P; ++p) {
    if (!e->active[p] || !e->stepped[p]) continue;
    const bool was_anchor = !e->mixed || e->anchor[p] || e->it[p] == 0;
    e->si[p] = e->hsi[p];
    if (!std::isfinite(e->si[p])) return fail(PNFAM_ENONFINITE, "non-finite residual");
    double smax = 0.0;
    for (int k = 0; k < nops; ++k) {
      double a = 0.0, b = 0.0;
      for (int ch = 0; ch < c->nchunk_c; ++ch) {
        a += e->cpart[((size_t)p * c->nchunk_c + ch) * 2 * nops + 2 * k];
        b += e->cpart[((size_t)p * c->nchunk_c + ch) * 2 * nops + 2 * k + 1];
      }
      const size_t i = (size_t)p * nops + k;
      e->pre[i] = e->sre[i]; e->pim[i] = e->sim[i];
      e->sre[i] = -a / pi;
      e->sim[i] = -b / pi;
      smax = std::max(smax, std::max(std::fabs(e->sre[i]), std::fabs(e->sim[i])));
    }
    // every strength value settled (always, unless opts.reserved[3] asks for it)
    bool settled = true;
    if (e->s_rel > 0.0) {
      for (int k = 0; k < nops && settled; ++k) {
        const size_t i = (size_t)p * nops + k;
        settled = std::fabs(e->sre[i] - e->pre[i]) <= e->s_rel * std::fabs(e->sre[i]) + 1e-13 * smax &&
                  std::fabs(e->sim[i] - e->pim[i]) <= e->s_rel * std::fabs(e->sim[i]) + 1e-13 * smax;
      }
    }
    const int it = ++e->it[p];
    engine_hist(e, p);
    const double si = e->si[p];
    // convergence (si < epsilon), held back while a strength value still moves
    auto accept = [&]() { return settled || ++e->extra[p] > pnfam_engine::EXTRA; };
    if (was_anchor) {
      if (si < o.convergence_epsilon && accept()) { engine_retire(e, p, it); continue; }
      if (e->mixed) { e->anchor[p] = 0; e->best[p] = si; e->since_best[p] = 0; }
    } else {
      double dm;
      std::memcpy(&dm, &e->hdmax[p], sizeof dm);
      const bool near = dm <= e->near * o.convergence_epsilon;
      if (si < o.convergence_epsilon && near && accept()) { engine_retire(e, p, it); continue; }
      if (si < e->best[p] * 0.5) { e->best[p] = si; e->since_best[p] = 0; } else { ++e->since_best[p]; }
      // the stagnation window doubles with every anchor it has triggered
      const bool stalled = e->since_best[p] >= (5 << std::min(e->nstall[p], 4)) &&
                           si <= pnfam_engine::FLOOR * dm;
      if (!near && (si < e->switch_si || stalled)) { e->anchor[p] = 1; e->nstall[p] += stalled; }
    }
    if (it == o.max_iter) engine_retire(e, p, -1);
  }
  return PNFAM_OK;
}

static int engine_nactive(const pnfam_engine* e) {
  int n = 0;
  for (int a : e->active) n += a;
  return n;
}

static int solve_impl(pnfam_ctx_t* c, int P, const double* re_w, const double* im_w,
                      const pnfam_solver_opts_t* o, const double* x0, double* re_S, double* im_S, int* iters,
                      double* si_out, double* hist, double* x_out) {
  g_err.clear();
  if (!c || !o || !re_w || !im_w || !re_S || !im_S || !iters || !si_out || P <= 0)
    return fail(PNFAM_EINVAL, "pnfam_gpu_solve: bad argument");
  if (c->engine) return fail(PNFAM_ESTATE, "pnfam_gpu_solve: the context's solve buffers belong to an engine");
  pnfam_engine e;
  int rc = engine_setup(&e, c, P, o);
  if (rc) { g_err = "pnfam_gpu_solve: " + g_err; return rc; }
  e.hist = hist;
  CK(cudaEventRecord(c->evt[0], c->stream));
  engine_admit(&e, P, re_w, im_w, nullptr);
  if (x0) {
    for (int p = 0; p < P; ++p)
      if (e.active[p] && (rc = engine_set_state(&e, p, x0 + (size_t)p * e.N))) return rc;
  }
  while (engine_nactive(&e) > 0) {
    if ((rc = engine_launch(&e, true)) || (rc = engine_finish(&e))) {
      cudaStreamSynchronize(c->stream64);
      cudaStreamSynchronize(c->stream);
      g_err = "pnfam_gpu_solve: " + g_err;
      return rc;
    }
  }
  CK(cudaEventRecord(c->evt[1], c->stream));
  CK(cudaEventSynchronize(c->evt[1]));
  {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->evt[0], c->evt[1]);
    c->total_ms = ms;
  }
  const int nops = c->nops;
  for (size_t k = 0; k < e.done.size(); ++k) {
    const int p = (int)e.done[k].tag;
    iters[p] = e.done[k].iters;
    si_out[p] = e.done[k].si;
    for (int q = 0; q < nops; ++q) {
      re_S[(size_t)p * nops + q] = e.done_re[k * nops + q];
      im_S[(size_t)p * nops + q] = e.done_im[k * nops + q];
    }
  }
  // the final state vectors (point p was admitted into slot p)
  if (x_out) {
    std::vector<double> v((size_t)P * e.N);
    CK(cudaMemcpy(v.data(), c->d_state.p, sizeof(double) * v.size(), cudaMemcpyDeviceToHost));
    for (int p = 0; p < P; ++p) state_to_ref(c->nq, c->nxy, v.data() + (size_t)p * e.N, x_out + (size_t)p * e.N);
  }
  return PNFAM_OK;
}

extern "C" int pnfam_gpu_solve(pnfam_ctx_t* c, int P, const double* re_w, const double* im_w,
                               const pnfam_solver_opts_t* o, double* re_S, double* im_S, int* iters,
                               double* si_out, double* hist) {
  return solve_impl(c, P, re_w, im_w, o, nullptr, re_S, im_S, iters, si_out, hist, nullptr);
}

extern "C" int pnfam_gpu_solve_state(pnfam_ctx_t* c, int P, const double* re_w, const double* im_w,
                                     const pnfam_solver_opts_t* o, const double* x0, double* re_S, double* im_S,
                                     int* iters, double* si_out, double* hist, double* x_out) {
  return solve_impl(c, P, re_w, im_w, o, x0, re_S, im_S, iters, si_out, hist, x_out);
}

extern "C" long long pnfam_gpu_state_size(const pnfam_ctx_t* c) {
  return c && c->have_op ? 2LL * c->nq * c->nxy : 0;
}

// ---- continuous-batching engine (C ABI) ----
extern "C" int pnfam_gpu_engine_create(pnfam_ctx_t* c, int slots, const pnfam_solver_opts_t* o,
                                       pnfam_engine_t** out) {
  g_err.clear();
  if (!c || !o || !out || slots <= 0) return fail(PNFAM_EINVAL, "pnfam_gpu_engine_create: bad argument");
  if (c->engine) return fail(PNFAM_ESTATE, "pnfam_gpu_engine_create: the context already has an engine");
  pnfam_engine* e = new pnfam_engine;
  int rc = engine_setup(e, c, slots, o);
  if (rc) { delete e; g_err = "pnfam_gpu_engine_create: " + g_err; return rc; }
  c->engine = e;
  *out = e;
  return PNFAM_OK;
}

extern "C" int pnfam_gpu_engine_admit(pnfam_engine_t* e, int n, const double* re_w, const double* im_w,
                                      const long long* tags) {
  g_err.clear();
  if (!e || n < 0 || (n > 0 && (!re_w || !im_w))) return -fail(PNFAM_EINVAL, "pnfam_gpu_engine_admit: bad argument");
  if (!e->c) return -fail(PNFAM_ESTATE, "pnfam_gpu_engine_admit: the context was freed");
  if (e->pending) return -fail(PNFAM_ESTATE, "pnfam_gpu_engine_admit: an evaluation is in flight");
  return engine_admit(e, n, re_w, im_w, tags);
}

extern "C" int pnfam_gpu_engine_launch(pnfam_engine_t* e) {
  g_err.clear();
  if (!e) return fail(PNFAM_EINVAL, "pnfam_gpu_engine_launch: NULL engine");
  if (!e->c) return fail(PNFAM_ESTATE, "pnfam_gpu_engine_launch: the context was freed");
  if (e->pending) return fail(PNFAM_ESTATE, "pnfam_gpu_engine_launch: an evaluation is in flight");
  const int rc = engine_launch(e, false);
  if (rc) {
    // nothing of a failed launch may stay in flight (the FP64 anchors' stream included)
    cudaStreamSynchronize(e->c->stream64);
    cudaStreamSynchronize(e->c->stream);
    e->pending = 0;
    g_err = "pnfam_gpu_engine_launch: " + g_err;
  }
  return rc;
}

extern "C" int pnfam_gpu_engine_finish(pnfam_engine_t* e, int maxout, long long* tags, double* re_S, double* im_S,
                                       int* iters, double* si, int* nout) {
  g_err.clear();
  if (!e || !nout || maxout < 0 || (maxout > 0 && (!tags || !re_S || !im_S || !iters || !si)))
    return fail(PNFAM_EINVAL, "pnfam_gpu_engine_finish: bad argument");
  if (!e->c) return fail(PNFAM_ESTATE, "pnfam_gpu_engine_finish: the context was freed");
  int rc = engine_finish(e);
  if (rc) { g_err = "pnfam_gpu_engine_finish: " + g_err; return rc; }
  const int nops = e->nops;
  const int n = std::min<int>(maxout, (int)e->done.size());
  for (int k = 0; k < n; ++k) {
    tags[k] = e->done[k].tag; iters[k] = e->done[k].iters; si[k] = e->done[k].si;
    for (int q = 0; q < nops; ++q) {
      re_S[(size_t)k * nops + q] = e->done_re[(size_t)k * nops + q];
      im_S[(size_t)k * nops + q] = e->done_im[(size_t)k * nops + q];
    }
  }
  e->done.erase(e->done.begin(), e->done.begin() + n);
  e->done_re.erase(e->done_re.begin(), e->done_re.begin() + (size_t)n * nops);
  e->done_im.erase(e->done_im.begin(), e->done_im.begin() + (size_t)n * nops);
  *nout = n;
  return PNFAM_OK;
}

extern "C" int pnfam_gpu_engine_active(const pnfam_engine_t* e) { return e ? engine_nactive(e) : 0; }

extern "C" int pnfam_gpu_engine_ready(const pnfam_engine_t* e) {
  if (!e || !e->c) return -PNFAM_EINVAL;
  if (!e->pending) return 1;
  const cudaError_t q = cudaEventQuery(e->c->evd);
  if (q == cudaSuccess) return 1;
  if (q == cudaErrorNotReady) return 0;
  return -PNFAM_ECUDA;
}

extern "C" void pnfam_gpu_engine_free(pnfam_engine_t* e) {
  if (!e) return;
  if (e->c) {
    cudaStreamSynchronize(e->c->stream64);   // anchor batches still in flight
    if (e->pending) cudaStreamSynchronize(e->c->stream);
    e->c->engine = nullptr;
  }
  delete e;
}

extern "C" int pnfam_gpu_calc_hamiltonian(pnfam_ctx_t* c, const double* re_rho_pn, const double* im_rho_pn,
                                          const double* re_kp, const double* im_kp, const double* re_rho_np,
                                          const double* im_rho_np, const double* re_km, const double* im_km,
                                          double* re_h_pn, double* im_h_pn, double* re_dp, double* im_dp,
                                          double* re_h_np, double* im_h_np, double* re_dm, double* im_dm) {
  g_err.clear();
  if (!c) return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian: NULL context");
  if (!c->have_op) return fail(PNFAM_ESTATE, "pnfam_gpu_calc_hamiltonian: call pnfam_gpu_set_operator first");
  const void* in[8] = {re_rho_pn, im_rho_pn, re_kp, im_kp, re_rho_np, im_rho_np, re_km, im_km};
  void* outp[8] = {re_h_pn, im_h_pn, re_dp, im_dp, re_h_np, im_h_np, re_dm, im_dm};
  for (int k = 0; k < 8; ++k)
    if (!in[k] || !outp[k]) return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian: NULL array");
  int rc = ensure_buffers(c, std::max(1, c->cap_P), std::max(1, c->cap_M));
  if (rc) return rc;
  const long long nxy = c->nxy;
  const size_t nb = sizeof(double) * nxy;
  // RSP quadrant q, plane pl at pl*4nxy + q*nxy (point 0): 0 rho_pn, 1 kappa+, 2 kappa-, 3 rho_np
  const int qin[8] = {0, 0, 1, 1, 3, 3, 2, 2};
  for (int k = 0; k < 8; ++k)
    CK(cudaMemcpyAsync(c->d_rsp.p + (k & 1) * 4 * nxy + qin[k] * nxy, in[k], nb, cudaMemcpyHostToDevice, c->stream));
  std::vector<int> one = {1};
  CK(cudaMemcpyAsync(c->d_active.p, one.data(), sizeof(int), cudaMemcpyHostToDevice, c->stream));
  DensCall d0, d1;
  d0.rho = c->d_rsp.p + 0 * nxy; d0.rho_sp = 8 * nxy; d0.rho_spl = 4 * nxy;
  d0.rcols = c->d_fc.p; d0.roffs = c->d_foff.p;
  d0.kap = c->d_rsp.p + 1 * nxy; d0.kap_sp = 8 * nxy; d0.kap_spl = 4 * nxy;
  d0.kcols = c->d_xtc.p; d0.koffs = c->d_xtoff.p;
  d1.rho = c->d_rsp.p + 3 * nxy; d1.rho_sp = 8 * nxy; d1.rho_spl = 4 * nxy;
  d1.rcols = c->d_fc.p; d1.roffs = c->d_foff.p;
  d1.kap = c->d_rsp.p + 2 * nxy; d1.kap_sp = 8 * nxy; d1.kap_spl = 4 * nxy;
  d1.kcols = c->d_ytc.p; d1.koffs = c->d_ytoff.p;
  const DevBasis B = c->devbasis<double>();
  const int* act = c->d_active.p;
  k_density_fp64<<<dim3((c->nghl + DRT - 1) / DRT, c->G, 2), 256, 0, c->stream>>>(B, d0, d1, c->G, c->d_dpart.p,
                                                                                 act);
  k_meanfield<<<dim3((c->nghl + 127) / 128, 2), 128, 0, c->stream>>>(B, c->G, c->d_dpart.p, c->d_mf.p, act);
  k_hproj_fp64<<<dim3((unsigned)c->htasks.size(), 1), 256, hproj_fp64_smem_bytes(), c->stream>>>(
      B, c->d_htasks.p, c->d_mf.p, c->d_hsp.p, nxy, act);
  CK(cudaGetLastError());
  const int qout[8] = {0, 0, 1, 1, 3, 3, 2, 2};
  for (int k = 0; k < 8; ++k)
    CK(cudaMemcpyAsync(outp[k], c->d_hsp.p + (k & 1) * 4 * nxy + qout[k] * nxy, nb, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return PNFAM_OK;
}

extern "C" int pnfam_gpu_calc_hamiltonian_mixed(pnfam_ctx_t* c, const double* re_rho_pn, const double* im_rho_pn,
                                                const double* re_kp, const double* im_kp, const double* re_rho_np,
                                                const double* im_rho_np, const double* re_km, const double* im_km,
                                                double* re_h_pn, double* im_h_pn, double* re_dp, double* im_dp,
                                                double* re_h_np, double* im_h_np, double* re_dm, double* im_dm) {
  g_err.clear();
  if (!c) return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_mixed: NULL context");
  if (!c->have_op) return fail(PNFAM_ESTATE, "pnfam_gpu_calc_hamiltonian_mixed: call pnfam_gpu_set_operator first");
  const void* in[8] = {re_rho_pn, im_rho_pn, re_kp, im_kp, re_rho_np, im_rho_np, re_km, im_km};
  void* outp[8] = {re_h_pn, im_h_pn, re_dp, im_dp, re_h_np, im_h_np, re_dm, im_dm};
  for (int k = 0; k < 8; ++k)
    if (!in[k] || !outp[k]) return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_mixed: NULL array");
  int rc = ensure_buffers(c, std::max(1, c->cap_P), std::max(1, c->cap_M));
  if (rc) return rc;
  c->cap_P = std::max(1, c->cap_P); c->cap_M = std::max(1, c->cap_M);
  if ((rc = ensure_buffers32(c, c->cap_P))) return rc;
  const long long nxy = c->nxy;
  const size_t nb = sizeof(double) * nxy;
  const int qin[8] = {0, 0, 1, 1, 3, 3, 2, 2};
  for (int k = 0; k < 8; ++k)
    CK(cudaMemcpyAsync(c->d_rsp.p + (k & 1) * 4 * nxy + qin[k] * nxy, in[k], nb, cudaMemcpyHostToDevice, c->stream));
  std::vector<int> one = {1}, zero = {0};
  CK(cudaMemcpyAsync(c->d_active.p, one.data(), sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d_actlist.p, zero.data(), sizeof(int), cudaMemcpyHostToDevice, c->stream));
  k_to_f32<<<1024, 256, 0, c->stream>>>(c->d_rsp.p, c->d_rsp32.p, 8 * nxy, 1, 0, nullptr);
  DensCallT<float> d0, d1;
  d0.rho = c->d_rsp32.p + 0 * nxy; d0.rho_sp = 8 * nxy; d0.rho_spl = 4 * nxy;
  d0.rcols = c->d_fc.p; d0.roffs = c->d_foff.p;
  d0.kap = c->d_rsp32.p + 1 * nxy; d0.kap_sp = 8 * nxy; d0.kap_spl = 4 * nxy;
  d0.kcols = c->d_xtc.p; d0.koffs = c->d_xtoff.p;
  d1.rho = c->d_rsp32.p + 3 * nxy; d1.rho_sp = 8 * nxy; d1.rho_spl = 4 * nxy;
  d1.rcols = c->d_fc.p; d1.roffs = c->d_foff.p;
  d1.kap = c->d_rsp32.p + 2 * nxy; d1.kap_sp = 8 * nxy; d1.kap_spl = 4 * nxy;
  d1.kcols = c->d_ytc.p; d1.koffs = c->d_ytoff.p;
  const DevBasisT<float> B = c->devbasis<float>();
  const int* act = c->d_active.p;
  if (c->tc_density) {
    DensTCArgs t0{d0.rho, d0.rho_sp, d0.rho_spl, d0.rcols, d0.roffs, d0.kap, d0.kap_sp, d0.kap_spl, d0.kcols, d0.koffs};
    DensTCArgs t1{d1.rho, d1.rho_sp, d1.rho_spl, d1.rcols, d1.roffs, d1.kap, d1.kap_sp, d1.kap_spl, d1.kcols, d1.koffs};
    if (!c->bchunks.empty())
      k_dens_bsplit<<<dim3((unsigned)c->bchunks.size(), 1), 256, 0, c->stream>>>(B, t0, t1, c->d_bchunks.p,
                                                                                c->d_actlist.p, c->d_bsplit.p,
                                                                                c->bstride);
    k_density_tc2<<<dim3((c->nghl + 31) / 32, c->G, 2), DTC2_THREADS, density_tc2_smem_bytes(), c->stream>>>(
        B, c->d_dunits0.p, (int)c->dunits[0].size(), c->d_dunits1.p, (int)c->dunits[1].size(), c->d_aphi.p,
        (int)c->achunks.size(), c->d_bsplit.p, c->bstride, c->G, c->d_actlist.p, c->d_dpart32.p, c->d_err.p);
  } else {
    k_density<float><<<dim3((c->nghl + DRT - 1) / DRT, c->G, 2), 256, density_smem_bytes<float>(), c->stream>>>(
        B, d0, d1, c->G, c->d_dpart32.p, act);
  }
  k_meanfield<float><<<dim3((c->nghl + 127) / 128, 2), 128, 0, c->stream>>>(B, c->G, c->d_dpart32.p, c->d_mf32.p, act);
  k_hproj_tc<<<dim3((unsigned)c->htasks_tc.size(), 1), HTC_THREADS, hproj_tc_smem_bytes(c->tc_npmax), c->stream>>>(
      B, c->d_htasks_tc.p, c->d_actlist.p, 1, c->tc_npmax, c->d_mf32.p, c->d_hphi.p, c->d_hsp32.p, nxy, c->d_err.p);
  k_to_f64<<<dim3(1024, 1), 256, 0, c->stream>>>(c->d_hsp32.p, c->d_hsp.p, 8 * nxy, 0, nullptr);
  CK(cudaGetLastError());
  const int qout[8] = {0, 0, 1, 1, 3, 3, 2, 2};
  for (int k = 0; k < 8; ++k)
    CK(cudaMemcpyAsync(outp[k], c->d_hsp.p + (k & 1) * 4 * nxy + qout[k] * nxy, nb, cudaMemcpyDeviceToHost, c->stream));
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, c->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (herr) {
    cudaMemsetAsync(c->d_err.p, 0, sizeof(int), c->stream);
    return fail(PNFAM_ECUDA, "pnfam_gpu_calc_hamiltonian_mixed: a wait on the tensor cores gave up");
  }
  return PNFAM_OK;
}

extern "C" int pnfam_gpu_set_occupations(pnfam_ctx_t* c, const double* fp, const double* fn) {
  g_err.clear();
  if (!c || (!fp) != (!fn)) return fail(PNFAM_EINVAL, "pnfam_gpu_set_occupations: pass both occupation arrays or neither");
  if (c->engine) return fail(PNFAM_ESTATE, "pnfam_gpu_set_occupations: an engine is using this context");
  if (!fp) {
    c->nq = 2;
  } else {
    for (int k = 0; k < c->dqp; ++k)
      if (!(fp[k] >= 0.0 && fp[k] <= 1.0 && fn[k] >= 0.0 && fn[k] <= 1.0))
        return fail(PNFAM_EINVAL, "pnfam_gpu_set_occupations: occupations must lie in [0, 1]");
    CK(upload(c->d_fp, fp, (size_t)c->dqp));
    CK(upload(c->d_fn, fn, (size_t)c->dqp));
    c->nq = 4;
  }
  c->have_op = false;   // the quadrant set changed: the operator is set again
  return PNFAM_OK;
}

static_assert(PNFAM_TASK_TERMS == PNFAM_MAXTERM, "task record layout");
extern "C" int pnfam_gpu_task_tables(int nb, const int* db, const int* num_spin_up, int beta_minus,
                                     const int* fcols, int statistical, int stage, double* out, int cap,
                                     int* ntask, long long* nxy, long long* scratch) {
  g_err.clear();
  if (!db || !num_spin_up || !fcols || !ntask || stage < 0 || stage > 3 || cap < 0 || (cap > 0 && !out))
    return fail(PNFAM_EINVAL, "pnfam_gpu_task_tables: bad argument");
  pnfam_ctx c;
  int rc = host_basis(&c, nb, 1, db, num_spin_up);
  if (rc) return rc;
  c.nq = statistical ? 4 : 2;
  if ((rc = host_structure(&c, beta_minus, fcols))) return rc;
  build_tasks(&c);
  const TaskList& tl = stage == 0 ? c.k1a : stage == 1 ? c.k1b : stage == 2 ? c.k2a : c.k2b;
  *ntask = (int)tl.tasks.size();
  if (nxy) *nxy = c.nxy;
  if (scratch) *scratch = c.tplane;
  const int n = std::min(cap, *ntask);
  for (int k = 0; k < n; ++k) {
    const GemmTask& t = tl.tasks[k];
    double* r = out + (size_t)k * PNFAM_TASK_RECORD;
    r[0] = t.M; r[1] = t.N; r[2] = t.K; r[3] = t.nterm; r[4] = t.cbuf; r[5] = (double)t.coff; r[6] = t.ldc;
    for (int i = 0; i < PNFAM_MAXTERM; ++i) {
      const GemmTerm& g = t.t[i];
      double* q = r + 7 + 10 * i;
      q[0] = g.abuf; q[1] = (double)g.aoff; q[2] = g.lda; q[3] = g.tA;
      q[4] = g.bbuf; q[5] = (double)g.boff; q[6] = g.ldb; q[7] = g.tB;
      q[8] = g.alpha[0]; q[9] = g.alpha[1];
    }
  }
  return PNFAM_OK;
}

extern "C" long long pnfam_gpu_nxy(const pnfam_ctx_t* c) { return c && c->have_op ? c->nxy : 0; }

extern "C" int pnfam_gpu_last_profile(const pnfam_ctx_t* c, double* stage_ms, int nstage, long long* launches) {
  if (!c) return fail(PNFAM_EINVAL, "pnfam_gpu_last_profile: NULL context");
  for (int k = 0; k < nstage && k < 8; ++k) stage_ms[k] = c->stage_ms[k];
  if (nstage > 8) stage_ms[8] = c->total_ms;
  if (nstage > 10) { stage_ms[9] = (double)c->pit64; stage_ms[10] = (double)c->pit32; }
  for (int k = 11; k < nstage && k < 16; ++k) stage_ms[k] = c->stage32_ms[k - 11];
  const double live[4] = {(double)c->live_n[0], c->live_ms[0], (double)c->live_n[1], c->live_ms[1]};
  for (int k = 16; k < nstage && k < 20; ++k) stage_ms[k] = live[k - 16];
  // the autotuner's choices: pg_min (2^30: the pair-tensor path never), the density
  // task span, and its host time in ms (0: not run)
  const double tune[3] = {(double)c->pg_min, (double)c->pg_kspan, c->tune_ms};
  for (int k = 20; k < nstage && k < 23; ++k) stage_ms[k] = tune[k - 20];
  if (launches) *launches = c->launches;
  return PNFAM_OK;
}

extern "C" void pnfam_gpu_free(pnfam_ctx_t* c) { delete c; }

extern "C" const char* pnfam_gpu_last_error(void) { return g_err.c_str(); }

// ---------------------------------------------------------------------------
// Allocation-free variant of pnfam_gpu_calc_hamiltonian
//
// For callers that cannot call cudaMalloc (a host code that owns all device
// memory through its own pool or mapped memory, or code running where device
// allocation is not allowed): the caller passes device pointers for every
// input and output, and all intermediates live in one file-scope device array
// of fixed size.  Every GPU that loads this library holds that array (about
// 12.5 MB) until the process exits.
// ---------------------------------------------------------------------------
namespace {
constexpr long long NA_MAX_NXY = 32768;   // FAM matrix elements (N_sh <= 12)
constexpr int NA_MAX_NGHL = 1600;         // mesh points (40 x 40)
constexpr int NA_MAX_DQP = 1024;          // basis states incl. time-reversed partners
constexpr int NA_MAX_NB = 64;             // blocks incl. time-reversed partners
constexpr int NA_MAX_HTASKS = 4096;       // field-projection tiles
constexpr int NA_G = 2;                   // block-row groups of the density kernel

constexpr size_t na_align(size_t n) { return (n + 255) / 256 * 256; }
constexpr size_t NA_RSP = na_align(sizeof(double) * 8 * NA_MAX_NXY);
constexpr size_t NA_HSP = na_align(sizeof(double) * 8 * NA_MAX_NXY);
constexpr size_t NA_DPART = na_align(sizeof(double) * 2 * NA_G * 2 * ND * NA_MAX_NGHL);
constexpr size_t NA_MF = na_align(sizeof(double) * 2 * NMF * 2 * NA_MAX_NGHL);
constexpr size_t NA_INTS = na_align(sizeof(int) * (6 * NA_MAX_NB + 1));
constexpr size_t NA_LONGS = na_align(sizeof(long long) * 3 * NA_MAX_NB);
constexpr size_t NA_NS = na_align(NA_MAX_DQP);
constexpr size_t NA_TASKS = na_align(sizeof(HTask) * NA_MAX_HTASKS);
constexpr size_t NA_BYTES = NA_RSP + NA_HSP + NA_DPART + NA_MF + NA_INTS + NA_LONGS + NA_NS + NA_TASKS;
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

namespace {
struct NaDevice {
  bool ready = false;
  unsigned char* ptr = nullptr;
};
NaDevice g_na_dev[64];
std::mutex g_na_mu;

// Once per device, with that device current: the device address of the
// scratch array (the host-side name is only a stand-in) and the kernel
// attribute the field projection needs.
int noalloc_setup(unsigned char** out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(PNFAM_ECUDA, "pnfam_gpu_calc_hamiltonian_noalloc: device index >= 64");
  std::lock_guard<std::mutex> lock(g_na_mu);
  NaDevice& d = g_na_dev[dev];
  if (!d.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(PNFAM_ECUDA, std::string("pnfam_gpu_calc_hamiltonian_noalloc: cudaGetSymbolAddress: ") +
                                   cudaGetErrorString(e));
    e = cudaFuncSetAttribute(k_hproj_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)hproj_fp64_smem_bytes());
    if (e != cudaSuccess)
      return fail(PNFAM_ECUDA, std::string("pnfam_gpu_calc_hamiltonian_noalloc: cudaFuncSetAttribute: ") +
                                   cudaGetErrorString(e));
    d.ptr = static_cast<unsigned char*>(p);
    d.ready = true;
  }
  *out = d.ptr;
  return PNFAM_OK;
}
}  // namespace

extern "C" int pnfam_gpu_calc_hamiltonian_noalloc(
    const pnfam_basis_t* basis, const double* d_phi, const double* d_wdcori, const pnfam_coupl_t* d_coupl,
    const int* fcols, const double* const* d_in, double* const* d_out, void* stream) {
  g_err.clear();
  if (!basis || !basis->db || !basis->num_spin_up || !basis->ns || !d_phi || !d_wdcori || !d_coupl || !fcols ||
      !d_in || !d_out)
    return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: NULL argument");
  for (int k = 0; k < 8; ++k)
    if (!d_in[k] || !d_out[k]) return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: NULL array");
  if (!d_coupl->crho || !d_coupl->cs || !d_coupl->cpair || !d_coupl->cspair)
    return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: NULL coupling array");
  const int nb = basis->nb, nghl = basis->nghl;
  if (nb <= 0 || nb % 2 || nghl <= 0)
    return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: nb must be positive and even, nghl positive");
  if (nb > NA_MAX_NB || nghl > NA_MAX_NGHL)
    return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: nb <= 64 and nghl <= 1600 are the limits");
  // host-side description (no device memory): reuse the solver's structure code
  pnfam_ctx c;
  c.nb = nb; c.nghl = nghl;
  c.db.assign(basis->db, basis->db + nb);
  c.nup.assign(basis->num_spin_up, basis->num_spin_up + nb);
  c.st.resize(nb); c.tr.resize(nb); c.uoff.resize(nb);
  int s = 0;
  long long mo = 0;
  for (int i = 0; i < nb; ++i) {
    if (c.db[i] < 0 || c.nup[i] < 0 || c.nup[i] > c.db[i])
      return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: bad block size or spin count");
    c.st[i] = s; s += c.db[i];
    c.uoff[i] = mo; mo += (long long)c.db[i] * c.db[i];
    c.tr[i] = i < nb / 2 ? i + nb / 2 : i - nb / 2;
  }
  if (s > NA_MAX_DQP) return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: dqp <= 1024 is the limit");
  c.dqp = s;
  std::vector<signed char> ns(s);
  for (int k = 0; k < s; ++k) {
    if (basis->ns[k] != 1 && basis->ns[k] != -1)
      return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: ns must be +-1");
    ns[k] = (signed char)basis->ns[k];
  }
  c.fc.assign(fcols, fcols + nb);
  for (int i = 0; i < nb; ++i)
    if (c.fc[i] < -1 || c.fc[i] >= nb) return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: fcols out of range");
  c.xc.assign(nb, -1); c.yc.assign(nb, -1); c.xtc.assign(nb, -1); c.ytc.assign(nb, -1);
  for (int i = 0; i < nb; ++i) {
    if (c.fc[i] >= 0) c.xc[i] = c.tr[c.fc[i]];
    c.yc[i] = c.fc[c.tr[i]];
  }
  for (int i = 0; i < nb; ++i) {
    if (c.xc[i] >= 0) { if (c.xtc[c.xc[i]] >= 0) return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: F is not one block per column"); c.xtc[c.xc[i]] = i; }
    if (c.yc[i] >= 0) { if (c.ytc[c.yc[i]] >= 0) return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: F is not one block per column"); c.ytc[c.yc[i]] = i; }
  }
  long long nf, nx, ny, nxt, nyt;
  c.foff = offsets(c.fc, c.db, &nf);
  c.xoff = offsets(c.xc, c.db, &nx);
  c.yoff = offsets(c.yc, c.db, &ny);
  c.xtoff = offsets(c.xtc, c.db, &nxt);
  c.ytoff = offsets(c.ytc, c.db, &nyt);
  if (nf != nx || nf != ny || nf != nxt || nf != nyt || nf == 0)
    return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: inconsistent block structure");
  if (nf > NA_MAX_NXY) return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: nxy <= 32768 is the limit");
  c.nxy = nf;
  build_tasks(&c);
  if ((int)c.htasks.size() > NA_MAX_HTASKS)
    return fail(PNFAM_EINVAL, "pnfam_gpu_calc_hamiltonian_noalloc: more than 4096 field-projection tiles");
  unsigned char* base = nullptr;
  int rc = noalloc_setup(&base);
  if (rc) return rc;
  // carve the scratch array
  double* rsp = reinterpret_cast<double*>(base);
  double* hsp = reinterpret_cast<double*>(base + NA_RSP);
  double* dpart = reinterpret_cast<double*>(base + NA_RSP + NA_HSP);
  double* mf = reinterpret_cast<double*>(base + NA_RSP + NA_HSP + NA_DPART);
  int* ints = reinterpret_cast<int*>(base + NA_RSP + NA_HSP + NA_DPART + NA_MF);
  long long* longs = reinterpret_cast<long long*>(base + NA_RSP + NA_HSP + NA_DPART + NA_MF + NA_INTS);
  signed char* dns = reinterpret_cast<signed char*>(base + NA_RSP + NA_HSP + NA_DPART + NA_MF + NA_INTS + NA_LONGS);
  HTask* dtasks = reinterpret_cast<HTask*>(base + NA_RSP + NA_HSP + NA_DPART + NA_MF + NA_INTS + NA_LONGS + NA_NS);
  std::vector<int> hints(6 * NA_MAX_NB + 1, 0);
  std::vector<long long> hlongs(3 * NA_MAX_NB, 0);
  for (int i = 0; i < nb; ++i) {
    hints[0 * NA_MAX_NB + i] = c.db[i];
    hints[1 * NA_MAX_NB + i] = c.st[i];
    hints[2 * NA_MAX_NB + i] = c.nup[i];
    hints[3 * NA_MAX_NB + i] = c.fc[i];
    hints[4 * NA_MAX_NB + i] = c.xtc[i];
    hints[5 * NA_MAX_NB + i] = c.ytc[i];
    hlongs[0 * NA_MAX_NB + i] = c.foff[i];
    hlongs[1 * NA_MAX_NB + i] = c.xtoff[i];
    hlongs[2 * NA_MAX_NB + i] = c.ytoff[i];
  }
  hints[6 * NA_MAX_NB] = 1;  // active flag of the single point
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t nbytes = sizeof(double) * nf;
  CK(cudaMemcpyAsync(ints, hints.data(), sizeof(int) * hints.size(), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(longs, hlongs.data(), sizeof(long long) * hlongs.size(), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(dns, ns.data(), (size_t)s, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(dtasks, c.htasks.data(), sizeof(HTask) * c.htasks.size(), cudaMemcpyHostToDevice, st));
  // inputs in the solver's quadrant layout: plane pl at pl*4nxy, quadrant q at q*nxy
  // (0 rho_pn, 1 kappa+, 2 kappa-, 3 rho_np)
  const int qin[8] = {0, 0, 1, 1, 3, 3, 2, 2};
  for (int k = 0; k < 8; ++k)
    CK(cudaMemcpyAsync(rsp + (k & 1) * 4 * nf + qin[k] * nf, d_in[k], nbytes, cudaMemcpyDeviceToDevice, st));
  DevBasis B;
  B.nb = nb; B.dqp = s; B.nghl = nghl;
  B.db = ints; B.st = ints + NA_MAX_NB; B.nup = ints + 2 * NA_MAX_NB; B.ns = dns;
  B.phi = d_phi; B.wdcori = d_wdcori;
  B.crho = d_coupl->crho; B.cs = d_coupl->cs; B.cpair = d_coupl->cpair; B.cspair = d_coupl->cspair;
  for (int i = 0; i < 12; ++i) B.sc[i] = d_coupl->scalars[i];
  const int* act = ints + 6 * NA_MAX_NB;
  DensCall d0, d1;
  d0.rho = rsp + 0 * nf; d0.rho_sp = 8 * nf; d0.rho_spl = 4 * nf;
  d0.rcols = ints + 3 * NA_MAX_NB; d0.roffs = longs;
  d0.kap = rsp + 1 * nf; d0.kap_sp = 8 * nf; d0.kap_spl = 4 * nf;
  d0.kcols = ints + 4 * NA_MAX_NB; d0.koffs = longs + NA_MAX_NB;
  d1.rho = rsp + 3 * nf; d1.rho_sp = 8 * nf; d1.rho_spl = 4 * nf;
  d1.rcols = ints + 3 * NA_MAX_NB; d1.roffs = longs;
  d1.kap = rsp + 2 * nf; d1.kap_sp = 8 * nf; d1.kap_spl = 4 * nf;
  d1.kcols = ints + 5 * NA_MAX_NB; d1.koffs = longs + 2 * NA_MAX_NB;
  k_density_fp64<<<dim3((nghl + DRT - 1) / DRT, NA_G, 2), 256, 0, st>>>(B, d0, d1, NA_G, dpart, act);
  k_meanfield<<<dim3((nghl + 127) / 128, 2), 128, 0, st>>>(B, NA_G, dpart, mf, act);
  k_hproj_fp64<<<dim3((unsigned)c.htasks.size(), 1), 256, hproj_fp64_smem_bytes(), st>>>(B, dtasks, mf, hsp, nf,
                                                                                       act);
  CK(cudaGetLastError());
  const int qout[8] = {0, 0, 1, 1, 3, 3, 2, 2};
  for (int k = 0; k < 8; ++k)
    CK(cudaMemcpyAsync(d_out[k], hsp + (k & 1) * 4 * nf + qout[k] * nf, nbytes, cudaMemcpyDeviceToDevice, st));
  CK(cudaStreamSynchronize(st));
  return PNFAM_OK;
}

// ---------------------------------------------------------------------------
// Finite-range two-body-current field (effective_2bc_extfield on the GPU)
// ---------------------------------------------------------------------------
namespace {
struct TbcDevice {      // device copies of the prepared tables, freed on scope exit
  DBuf<double> jz, xr, cp, prho, zbuf, acc;
  DBuf<int> tq, poff, pz, gq, goff, el;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  ~TbcDevice() {
    jz.release(); xr.release(); cp.release(); prho.release(); zbuf.release(); acc.release();
    tq.release(); poff.release(); pz.release(); gq.release(); goff.release(); el.release();
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
  }
};
}  // namespace

extern "C" int pnfam_gpu_2bc_field(const pnfam_2bc_input_t* in, double* pieces, double* stats) {
  g_err.clear();
  if (!in || !pieces || !in->block_size || !in->nz || !in->nr || !in->nl || !in->ns || !in->rk_n || !in->rk_p ||
      !in->op_cols || !in->op_offsets || in->nxy <= 0)
    return fail(PNFAM_EINVAL, "pnfam_gpu_2bc_field: missing input");
  const auto h0 = std::chrono::steady_clock::now();
  tbc::Input ti{in->ntx, in->nbx, in->block_size, in->nz, in->nr, in->nl, in->ns, in->bz, in->bp, in->rk_n, in->rk_p,
                in->K, in->beta_minus ? 1 : 0, in->use_p ? 1 : 0, in->op_cols, in->op_offsets, in->nxy};
  tbc::Prepared P;
  const std::string why = tbc::prepare(ti, P);
  if (!why.empty()) return fail(PNFAM_EINVAL, "pnfam_gpu_2bc_field: " + why);
  if ((long long)P.out_index.size() != in->nxy)
    return fail(PNFAM_EINVAL, "pnfam_gpu_2bc_field: operator block structure does not match nxy");
  const double prep_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - h0).count();

  TbcDevice d;
  CK(upload(d.jz, P.jz.data(), P.jz.size()));
  CK(upload(d.xr, P.xr.data(), P.xr.size()));
  CK(upload(d.cp, P.cp.data(), P.cp.size()));
  CK(upload(d.tq, P.tq.data(), P.tq.size()));
  CK(upload(d.poff, P.poff.data(), P.poff.size()));
  CK(upload(d.pz, P.pz.data(), P.pz.size()));
  CK(upload(d.prho, P.prho.data(), P.prho.size()));
  CK(upload(d.gq, P.gq.data(), P.gq.size()));
  CK(upload(d.goff, P.goff.data(), P.goff.size()));
  CK(upload(d.el, P.el.data(), P.el.size()));
  tbc::View v = tbc::view_of(ti, P);
  v.jz = d.jz.p; v.xr = d.xr.p; v.cp = d.cp.p; v.tq = d.tq.p; v.poff = d.poff.p; v.pz = d.pz.p; v.prho = d.prho.p;
  v.gq = d.gq.p; v.goff = d.goff.p; v.el = d.el.p;
  const int NZ = P.nzx + 1;
  const long long nzt = (long long)NZ * NZ * v.nt;
  CK(dalloc(d.zbuf, (size_t)nzt * tbc::NQ * tbc::NCG));
  CK(dalloc(d.acc, (size_t)in->nxy * 6));
  CK(cudaMemset(d.acc.p, 0, (size_t)in->nxy * 6 * sizeof(double)));
  v.zbuf = d.zbuf.p; v.acc = d.acc.p;
  for (auto& e : d.ev) CK(cudaEventCreate(&e));

  CK(cudaEventRecord(d.ev[0], 0));
  const long long total = nzt * tbc::NCG;
  const int zgrid = (int)std::min<long long>((total + 255) / 256, 152LL * 64);
  tbc::k_tbc_z<<<zgrid, 256>>>(v, total);
  CK(cudaGetLastError());
  CK(cudaEventRecord(d.ev[1], 0));
  CK(cudaFuncSetAttribute(tbc::k_tbc_field, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tbc::TBC_SMEM));
  if (v.ngroups > 0) tbc::k_tbc_field<<<v.ngroups, tbc::TBC_THREADS, tbc::TBC_SMEM>>>(v);
  CK(cudaGetLastError());
  CK(cudaEventRecord(d.ev[2], 0));
  std::vector<double> acc((size_t)in->nxy * 6);
  CK(cudaMemcpy(acc.data(), d.acc.p, acc.size() * sizeof(double), cudaMemcpyDeviceToHost));
  float ms1 = 0.f, ms2 = 0.f;
  CK(cudaEventElapsedTime(&ms1, d.ev[0], d.ev[1]));
  CK(cudaEventElapsedTime(&ms2, d.ev[1], d.ev[2]));
  tbc::scatter(P, acc.data(), in->nxy, pieces);
  for (long long i = 0; i < 6 * in->nxy; ++i)
    if (!std::isfinite(pieces[i])) return fail(PNFAM_ENONFINITE, "pnfam_gpu_2bc_field: non-finite field element");
  if (stats) {
    stats[0] = prep_ms; stats[1] = ms1; stats[2] = ms2;
    stats[3] = v.nt; stats[4] = v.ngroups; stats[5] = (double)(P.pz.size() / 2);
  }
  return PNFAM_OK;
}

// ---------------------------------------------------------------------------
// HFB reconstruction kernels (basis functions, HFB matrices, batched symmetric
// eigensolver, local densities)
// ---------------------------------------------------------------------------
namespace {
struct HfbBufs {
  DBuf<double> d[8];
  DBuf<int> i[4];
  DBuf<size_t> z[2];
  DBuf<long long> l[1];
  ~HfbBufs() {
    for (auto& b : d) b.release();
    for (auto& b : i) b.release();
    for (auto& b : z) b.release();
    for (auto& b : l) b.release();
  }
};
int grid_for(long long n, int threads) { return (int)std::min<long long>((n + threads - 1) / threads, 152LL * 32); }
}  // namespace

extern "C" int pnfam_gpu_hfb_basis(int ngh, int ngl, const double* xh, const double* wh, const double* xl,
                                   const double* wl, double bz, double bp, int nt, const int* nr, const int* nz,
                                   const int* nl, double* out) {
  g_err.clear();
  if (ngh <= 0 || ngl <= 0 || nt <= 0 || !xh || !wh || !xl || !wl || !nr || !nz || !nl || !out || bz <= 0 || bp <= 0)
    return fail(PNFAM_EINVAL, "pnfam_gpu_hfb_basis: bad arguments");
  HfbBufs B;
  const size_t nghl = (size_t)ngh * ngl;
  CK(upload(B.d[0], xh, ngh)); CK(upload(B.d[1], wh, ngh)); CK(upload(B.d[2], xl, ngl)); CK(upload(B.d[3], wl, ngl));
  CK(upload(B.i[0], nr, nt)); CK(upload(B.i[1], nz, nt)); CK(upload(B.i[2], nl, nt));
  CK(dalloc(B.d[4], 4 * nghl * nt));
  hfbk::BasisView b{ngh, ngl, nt, B.d[0].p, B.d[1].p, B.d[2].p, B.d[3].p, bz, bp, B.i[0].p, B.i[1].p, B.i[2].p, B.d[4].p};
  hfbk::k_hfb_basis<<<grid_for((long long)nt * nghl, 256), 256>>>(b);
  CK(cudaGetLastError());
  CK(cudaMemcpy(out, B.d[4].p, 4 * nghl * nt * sizeof(double), cudaMemcpyDeviceToHost));
  return PNFAM_OK;
}

extern "C" int pnfam_gpu_hfb_matrices(int nb, const int* block_size, int nghl, const int* ns, const double* basis,
                                      const double* y, const double* xlam, const double* xlap, const double* fields,
                                      double* out) {
  g_err.clear();
  if (nb <= 0 || nghl <= 0 || !block_size || !ns || !basis || !y || !xlam || !xlap || !fields || !out)
    return fail(PNFAM_EINVAL, "pnfam_gpu_hfb_matrices: bad arguments");
  std::vector<int> bstart(nb + 1, 0);
  for (int ib = 0; ib < nb; ++ib) {
    if (block_size[ib] <= 0) return fail(PNFAM_EINVAL, "pnfam_gpu_hfb_matrices: empty block");
    bstart[ib + 1] = bstart[ib] + block_size[ib];
  }
  const int nt = bstart[nb];
  std::vector<size_t> moff(2 * (size_t)nb);
  std::vector<int> items;
  size_t tot = 0;
  for (int ib = 0; ib < nb; ++ib) {
    const int nd = block_size[ib];
    for (int it = 0; it < 2; ++it) {
      moff[2 * ib + it] = tot;
      tot += 2 * (size_t)nd * nd;
      for (int i = 0; i < nd; ++i)
        for (int j = 0; j <= i; ++j) items.insert(items.end(), {it, ib, i, j});
    }
  }
  HfbBufs B;
  CK(upload(B.i[0], bstart.data(), bstart.size()));
  CK(upload(B.i[1], ns, nt));
  CK(upload(B.i[2], items.data(), items.size()));
  CK(upload(B.d[0], basis, 4 * (size_t)nt * nghl));
  CK(upload(B.d[1], y, nghl));
  CK(upload(B.d[2], xlam, nb));
  CK(upload(B.d[3], xlap, nb));
  CK(upload(B.d[4], fields, 2 * (size_t)hfbk::NFIELD * nghl));
  CK(upload(B.z[0], moff.data(), moff.size()));
  CK(dalloc(B.d[5], tot));
  hfbk::MatView m{nb, nt, nghl, B.i[0].p, B.i[1].p, B.d[0].p, B.d[1].p, B.d[2].p, B.d[3].p, B.d[4].p, B.z[0].p,
                  B.d[5].p};
  const int nitems = (int)(items.size() / 4);
  hfbk::k_hfb_matrices<<<grid_for(nitems, 128), 128>>>(m, B.i[2].p, nitems);
  CK(cudaGetLastError());
  CK(cudaMemcpy(out, B.d[5].p, tot * sizeof(double), cudaMemcpyDeviceToHost));
  return PNFAM_OK;
}

extern "C" int pnfam_gpu_sym_eigen(int nmat, const int* dims, const double* a, const double* v0, double* w, double* v,
                                   int* sweeps) {
  g_err.clear();
  if (nmat <= 0 || !dims || !a || !w || !v) return fail(PNFAM_EINVAL, "pnfam_gpu_sym_eigen: bad arguments");
  std::vector<long long> off(nmat + 1, 0);
  int maxn = 0;
  for (int k = 0; k < nmat; ++k) {
    if (dims[k] <= 0 || dims[k] > hfbk::JAC_MAXN)
      return fail(PNFAM_EINVAL, "pnfam_gpu_sym_eigen: matrix size outside 1.." + std::to_string(hfbk::JAC_MAXN));
    off[k + 1] = off[k] + (long long)dims[k] * dims[k];
    maxn = std::max(maxn, dims[k]);
  }
  // device buffers kept for the process (grow-only): the particle-number loop calls
  // this tens of times per ground state
  static std::mutex mu;
  static HfbBufs* pool = new HfbBufs;
  static int smem_set = 0;
  std::lock_guard<std::mutex> lock(mu);
  HfbBufs& B = *pool;
  CK(upload(B.d[0], a, (size_t)off[nmat]));
  CK(dalloc(B.d[1], (size_t)off[nmat]));
  if (v0) CK(upload(B.d[2], v0, (size_t)off[nmat]));
  CK(upload(B.l[0], off.data(), off.size()));
  CK(upload(B.i[0], dims, nmat));
  CK(dalloc(B.i[1], nmat));
  const int smem_n = maxn <= hfbk::JAC_SMEM_N ? maxn : 0;
  const size_t smem = (size_t)smem_n * smem_n * sizeof(double);
  if (!smem_set) {
    CK(cudaFuncSetAttribute(hfbk::k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)((size_t)hfbk::JAC_SMEM_N * hfbk::JAC_SMEM_N * sizeof(double))));
    smem_set = 1;
  }
  hfbk::k_jacobi<<<nmat, hfbk::JAC_THREADS, smem>>>(B.d[0].p, B.d[1].p, v0 ? B.d[2].p : nullptr, B.l[0].p, B.i[0].p,
                                                   B.i[1].p, smem_n);
  CK(cudaGetLastError());
  std::vector<double> ha((size_t)off[nmat]), hv((size_t)off[nmat]);
  std::vector<int> st(nmat);
  CK(cudaMemcpy(ha.data(), B.d[0].p, ha.size() * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hv.data(), B.d[1].p, hv.size() * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(st.data(), B.i[1].p, nmat * sizeof(int), cudaMemcpyDeviceToHost));
  // eigenvalues ascending, eigenvectors as columns in the same order
  long long wo = 0;
  for (int k = 0; k < nmat; ++k) {
    const int n = dims[k];
    if (st[k] < 0) return fail(PNFAM_ENONFINITE, "pnfam_gpu_sym_eigen: Jacobi did not converge for matrix " +
                                                 std::to_string(k));
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    const double* A = ha.data() + off[k];
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return A[(size_t)x * n + x] < A[(size_t)y * n + y]; });
    for (int c = 0; c < n; ++c) {
      w[wo + c] = A[(size_t)ord[c] * n + ord[c]];
      for (int i = 0; i < n; ++i) v[off[k] + (size_t)i * n + c] = hv[off[k] + (size_t)ord[c] * n + i];
    }
    wo += n;
    if (sweeps) sweeps[k] = st[k];
  }
  return PNFAM_OK;
}

extern "C" int pnfam_gpu_hfb_densities(int nb, const int* block_size, int nghl, const int* ns, const double* basis,
                                       const double* y, const double* xlam, const double* xlap, const double* W,
                                       const double* U, const double* f, double* out) {
  g_err.clear();
  if (nb <= 0 || nghl <= 0 || !block_size || !ns || !basis || !y || !xlam || !xlap || !W || !out || (!U) != (!f))
    return fail(PNFAM_EINVAL, "pnfam_gpu_hfb_densities: bad arguments");
  std::vector<int> bstart(nb + 1, 0);
  std::vector<size_t> woff(nb);
  size_t tot = 0;
  for (int ib = 0; ib < nb; ++ib) {
    if (block_size[ib] <= 0) return fail(PNFAM_EINVAL, "pnfam_gpu_hfb_densities: empty block");
    bstart[ib + 1] = bstart[ib] + block_size[ib];
    woff[ib] = tot;
    tot += (size_t)block_size[ib] * block_size[ib];
  }
  const int nt = bstart[nb];
  HfbBufs B;
  CK(upload(B.i[0], bstart.data(), bstart.size()));
  CK(upload(B.i[1], ns, nt));
  CK(upload(B.d[0], basis, 4 * (size_t)nt * nghl));
  CK(upload(B.d[1], y, nghl));
  CK(upload(B.d[2], xlam, nb));
  CK(upload(B.d[3], xlap, nb));
  CK(upload(B.d[4], W, tot));
  if (U) { CK(upload(B.d[5], U, tot)); CK(upload(B.d[6], f, nt)); }
  CK(upload(B.z[0], woff.data(), woff.size()));
  CK(dalloc(B.d[7], 3 * (size_t)nghl));
  CK(cudaMemset(B.d[7].p, 0, 3 * (size_t)nghl * sizeof(double)));
  hfbk::DensView d{nb, nt, nghl, B.i[0].p, B.i[1].p, B.d[0].p, B.d[1].p, B.d[2].p, B.d[3].p, B.z[0].p, B.d[4].p,
                   U ? B.d[5].p : nullptr, U ? B.d[6].p : nullptr, B.d[7].p};
  hfbk::k_hfb_densities<<<grid_for((long long)nb * nghl, 128), 128>>>(d);
  CK(cudaGetLastError());
  CK(cudaMemcpy(out, B.d[7].p, 3 * (size_t)nghl * sizeof(double), cudaMemcpyDeviceToHost));
  return PNFAM_OK;
}
