// Test infrastructure: runs the per-item functions of the GPU two-body-current
// contraction (pynfam_gb300/csrc/tbc.cuh) serially on the host, in the order the
// two kernels cover their items, so that their arithmetic and indexing can be
// checked on a machine without a GPU.  Built by tests/test_finite_range_2bc.py
// with g++; never part of the library.
#include "../include/pnfam_gpu.h"
#include "../pynfam_gb300/csrc/tbc.cuh"

extern "C" int tbc_host_field(const pnfam_2bc_input_t* in, double* pieces, double* stats) {
  tbc::Input ti{in->ntx, in->nbx, in->block_size, in->nz, in->nr, in->nl, in->ns, in->bz, in->bp, in->rk_n, in->rk_p,
                in->K, in->beta_minus ? 1 : 0, in->use_p ? 1 : 0, in->op_cols, in->op_offsets, in->nxy};
  tbc::Prepared P;
  if (!tbc::prepare(ti, P).empty()) return 1;
  if ((long long)P.out_index.size() != in->nxy) return 2;
  tbc::View v = tbc::view_of(ti, P);
  const int NZ = P.nzx + 1;
  std::vector<double> zbuf((size_t)NZ * NZ * v.nt * tbc::NQ * tbc::NCG), acc((size_t)in->nxy * 6, 0.0);
  v.zbuf = zbuf.data();
  v.acc = acc.data();
  for (int zac = 0; zac < NZ * NZ; ++zac)
    for (int t = 0; t < v.nt; ++t)
      for (int cg = 0; cg < tbc::NCG; ++cg) tbc::stage1_item(v, zac, t, cg);
  std::vector<double> jd(tbc::NCG), je(tbc::NCG);
  for (int grp = 0; grp < v.ngroups; ++grp)
    for (int t = 0; t < v.nt; ++t)
      for (int br = 0; br < 2; ++br) {
        if (!tbc::stage2_jr(v, grp, t, br, 0, jd.data())) continue;
        tbc::stage2_jr(v, grp, t, br, 1, je.data());
        for (int e = v.goff[grp]; e < v.goff[grp + 1]; ++e)
          tbc::stage2_elem(v, grp, e, t, br, jd.data(), je.data(), acc.data() + (size_t)e * 6);
      }
  tbc::scatter(P, acc.data(), in->nxy, pieces);
  if (stats) {
    stats[3] = v.nt; stats[4] = v.ngroups; stats[5] = (double)(P.pz.size() / 2);
  }
  return 0;
}
