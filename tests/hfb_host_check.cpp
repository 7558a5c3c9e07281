// Test infrastructure: the per-item functions of the GPU HFB reconstruction
// (pynfam_gb300/csrc/hfb.cuh) run serially on the host, in the order the kernels
// cover their items (the Jacobi rounds in the kernel's step order), behind the same
// signatures as the library's entry points.  Built by tests/test_hfb_device.py with
// g++; never part of the library.
#include <algorithm>
#include <vector>

#include "../pynfam_gb300/csrc/hfb.cuh"

extern "C" int pnfam_gpu_hfb_basis(int ngh, int ngl, const double* xh, const double* wh, const double* xl,
                                   const double* wl, double bz, double bp, int nt, const int* nr, const int* nz,
                                   const int* nl, double* out) {
  hfbk::BasisView b{ngh, ngl, nt, xh, wh, xl, wl, bz, bp, nr, nz, nl, out};
  for (int t = 0; t < nt; ++t)
    for (int r = 0; r < ngh * ngl; ++r) hfbk::basis_item(b, t, r);
  return 0;
}

extern "C" int pnfam_gpu_hfb_matrices(int nb, const int* block_size, int nghl, const int* ns, const double* basis,
                                      const double* y, const double* xlam, const double* xlap, const double* fields,
                                      double* out) {
  std::vector<int> bstart(nb + 1, 0);
  for (int ib = 0; ib < nb; ++ib) bstart[ib + 1] = bstart[ib] + block_size[ib];
  std::vector<size_t> moff(2 * (size_t)nb);
  size_t tot = 0;
  for (int ib = 0; ib < nb; ++ib)
    for (int it = 0; it < 2; ++it) { moff[2 * ib + it] = tot; tot += 2 * (size_t)block_size[ib] * block_size[ib]; }
  hfbk::MatView m{nb, bstart[nb], nghl, bstart.data(), ns, basis, y, xlam, xlap, fields, moff.data(), out};
  for (int ib = 0; ib < nb; ++ib)
    for (int it = 0; it < 2; ++it)
      for (int i = 0; i < block_size[ib]; ++i)
        for (int j = 0; j <= i; ++j) hfbk::matrix_item(m, it, ib, i, j);
  return 0;
}

extern "C" int pnfam_gpu_sym_eigen(int nmat, const int* dims, const double* a, const double* v0, double* w, double* v,
                                   int* sweeps) {
  long long off = 0, wo = 0;
  for (int k = 0; k < nmat; ++k) {
    const int n = dims[k], m = n + (n & 1);
    std::vector<double> A(a + off, a + off + (size_t)n * n), V((size_t)n * n, 0.0);
    if (v0) {
      // the kernel's start: T = A V0, A = V0^T T, symmetrised, V = V0
      const double* q0 = v0 + off;
      std::vector<double> T((size_t)n * n);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          double t = 0.0;
          for (int kk = 0; kk < n; ++kk) t += A[(size_t)i * n + kk] * q0[(size_t)kk * n + j];
          T[(size_t)i * n + j] = t;
        }
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          double t = 0.0;
          for (int kk = 0; kk < n; ++kk) t += q0[(size_t)kk * n + i] * T[(size_t)kk * n + j];
          A[(size_t)i * n + j] = t;
        }
      for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
          const double x = 0.5 * (A[(size_t)i * n + j] + A[(size_t)j * n + i]);
          A[(size_t)i * n + j] = A[(size_t)j * n + i] = x;
        }
      for (int c = 0; c < n; ++c)
        for (int i = 0; i < n; ++i) V[(size_t)c * n + i] = q0[(size_t)i * n + c];   // transposed
    } else {
      for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
    }
    double nrm = 0.0;
    for (double x : A) nrm += x * x;
    nrm = std::sqrt(nrm);
    int sweep = 0;
    bool done = n <= 1;
    std::vector<int> pp(m / 2), qq(m / 2);
    std::vector<double> cc(m / 2), ss(m / 2);
    for (; sweep < hfbk::JAC_MAX_SWEEPS && !done; ++sweep) {
      double o = 0.0;
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
          if (i != j) o += A[(size_t)i * n + j] * A[(size_t)i * n + j];
      if (std::sqrt(o) <= hfbk::JAC_TOL * nrm) { done = true; break; }
      for (int r = 0; r < m - 1; ++r) {
        for (int kk = 0; kk < m / 2; ++kk) {
          int p, q;
          hfbk::rr_pair(r, kk, m, &p, &q);
          double c = 1.0, s = 0.0;
          if (q < n) hfbk::jacobi_cs(A[(size_t)p * n + p], A[(size_t)q * n + q], A[(size_t)p * n + q], &c, &s);
          pp[kk] = p; qq[kk] = q < n ? q : -1; cc[kk] = c; ss[kk] = s;
        }
        for (int kk = 0; kk < m / 2; ++kk)
          if (qq[kk] >= 0 && ss[kk] != 0.0)
            for (int j = 0; j < n; ++j) hfbk::jacobi_row(A.data(), n, pp[kk], qq[kk], cc[kk], ss[kk], j);
        for (int kk = 0; kk < m / 2; ++kk)
          if (qq[kk] >= 0 && ss[kk] != 0.0)
            for (int i = 0; i < n; ++i) {
              hfbk::jacobi_col(A.data(), n, pp[kk], qq[kk], cc[kk], ss[kk], i);
              hfbk::jacobi_vt(V.data(), n, pp[kk], qq[kk], cc[kk], ss[kk], i);
            }
        for (int kk = 0; kk < m / 2; ++kk)
          if (qq[kk] >= 0 && ss[kk] != 0.0) hfbk::jacobi_zero(A.data(), n, pp[kk], qq[kk]);
      }
    }
    if (!done) return 4;
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return A[(size_t)x * n + x] < A[(size_t)y * n + y]; });
    for (int c = 0; c < n; ++c) {
      w[wo + c] = A[(size_t)ord[c] * n + ord[c]];
      for (int i = 0; i < n; ++i) v[off + (size_t)i * n + c] = V[(size_t)ord[c] * n + i];
    }
    if (sweeps) sweeps[k] = sweep;
    off += (long long)n * n;
    wo += n;
  }
  return 0;
}

extern "C" int pnfam_gpu_hfb_densities(int nb, const int* block_size, int nghl, const int* ns, const double* basis,
                                       const double* y, const double* xlam, const double* xlap, const double* W,
                                       const double* U, const double* f, double* out) {
  std::vector<int> bstart(nb + 1, 0);
  std::vector<size_t> woff(nb);
  size_t tot = 0;
  for (int ib = 0; ib < nb; ++ib) {
    bstart[ib + 1] = bstart[ib] + block_size[ib];
    woff[ib] = tot;
    tot += (size_t)block_size[ib] * block_size[ib];
  }
  for (int i = 0; i < 3 * nghl; ++i) out[i] = 0.0;
  hfbk::DensView d{nb, bstart[nb], nghl, bstart.data(), ns, basis, y, xlam, xlap, woff.data(), W, U, f, out};
  for (int ib = 0; ib < nb; ++ib)
    for (int r = 0; r < nghl; ++r) {
      double acc[3];
      hfbk::density_item(d, ib, r, acc);
      for (int c = 0; c < 3; ++c) out[(size_t)c * nghl + r] += acc[c];
    }
  return 0;
}

extern "C" const char* pnfam_gpu_last_error(void) { return "host harness"; }
