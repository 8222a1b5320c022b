// Mesh preparation on the host: validation, the reference's mesh metrics
// (calc_mesh_metrics, mesh.c:19-83), cell renumbering (Morton or reverse
// Cuthill-McKee), face ordering and the device upload in the layouts the
// kernels read.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <tuple>
#include <cstring>
#include <numeric>
#include <queue>

#include "context.h"
#include "implicit.h"

namespace fv3d {

namespace {

uint64_t spread3(uint64_t v) {  // 21 bits -> every third bit
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

std::vector<int> morton_order(int nc, const double* x) {
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = 0; i < nc; ++i)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], x[3 * i + d]);
      hi[d] = std::max(hi[d], x[3 * i + d]);
    }
  std::vector<uint64_t> key(nc);
  for (int i = 0; i < nc; ++i) {
    uint64_t k = 0;
    for (int d = 0; d < 3; ++d) {
      double s = (hi[d] > lo[d]) ? (x[3 * i + d] - lo[d]) / (hi[d] - lo[d]) : 0.0;
      uint64_t q = (uint64_t)std::min(2097151.0, std::max(0.0, std::floor(s * 2097151.0)));
      k |= spread3(q) << d;
    }
    key[i] = k;
  }
  std::vector<int> order(nc);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
  return order;
}

// reverse Cuthill-McKee on the cell adjacency (interior faces)
std::vector<int> rcm_order(int nc, const std::vector<std::vector<int>>& adj) {
  std::vector<int> order;
  order.reserve(nc);
  std::vector<char> seen(nc, 0);
  std::vector<int> deg(nc);
  for (int i = 0; i < nc; ++i) deg[i] = (int)adj[i].size();
  std::vector<int> by_deg(nc);
  std::iota(by_deg.begin(), by_deg.end(), 0);
  std::stable_sort(by_deg.begin(), by_deg.end(), [&](int a, int b) { return deg[a] < deg[b]; });
  for (int start : by_deg) {
    if (seen[start]) continue;
    std::queue<int> q;
    q.push(start);
    seen[start] = 1;
    while (!q.empty()) {
      int c = q.front();
      q.pop();
      order.push_back(c);
      std::vector<int> nb;
      for (int o : adj[c])
        if (!seen[o]) { seen[o] = 1; nb.push_back(o); }
      std::stable_sort(nb.begin(), nb.end(), [&](int a, int b) { return deg[a] < deg[b]; });
      for (int o : nb) q.push(o);
    }
  }
  std::reverse(order.begin(), order.end());
  return order;
}

}  // namespace

fv3d_status prepare_mesh(Ctx& ctx, const fv3d_mesh_arrays& m) {
  ctx.mesh_ready = ctx.state_ready = ctx.residual_valid = false;
  ctx.release_graphs();
  // the implicit solver's buffers and face data belong to the old mesh
  delete ctx.implicit;
  ctx.implicit = nullptr;
  const int nc = m.n_cells, nf = m.n_faces, nb = m.n_boundaries, mcf = m.max_cell_faces;
  if (nc <= 0 || nf <= 0 || nb < 0 || mcf <= 0 || mcf > 8 || m.n_regions <= 0 ||
      m.n_regions > MAX_REGIONS)
    return ctx.fail(FV3D_ERR_INVALID_ARG, "bad mesh sizes (cells %d faces %d boundaries %d max faces %d regions %d)",
                    nc, nf, nb, mcf, m.n_regions);
  // face slots carry (face << 1) | side and the mixed path's other-side
  // index (record << 1) | side in an int: faces and face-side records
  // (max_cell_faces x cells rounded up to whole tiles, plus boundaries)
  // must stay below 2^30
  constexpr long long kIndexLimit = 1LL << 30;
  const long long slots = (mcf <= 4) ? 4 : (mcf <= 6 ? 6 : 8);   // the padded slot stride below
  if (nf >= kIndexLimit || slots * ((nc + kTile - 1LL) / kTile * kTile) + nb >= kIndexLimit)
    return ctx.fail(FV3D_ERR_UNSUPPORTED, "mesh too large for 31-bit face-side indices (cells %d faces %d max faces %d)",
                    nc, nf, mcf);
  if (!m.cell_x || !m.cell_volume || !m.cell_dx || !m.cell_n_faces || !m.cell_faces || !m.face_cells ||
      !m.face_boundary || !m.face_area || !m.face_lambda || !m.face_x || !m.face_n || !m.face_t1 ||
      !m.face_t2 || (nb > 0 && (!m.boundary_id || !m.boundary_face)) || !m.region_is_boundary)
    return ctx.fail(FV3D_ERR_INVALID_ARG, "missing mesh array");
  // ---- validation (a corrupt mesh is rejected here, never run) ----
  std::vector<int> fc1(nf);
  int n_bfaces = 0;
  for (int f = 0; f < nf; ++f) {
    int a = m.face_cells[2 * f], b = m.face_cells[2 * f + 1], bf = m.face_boundary[f];
    if (a < 0 || a >= nc) return ctx.fail(FV3D_ERR_BOUNDS, "face %d: cell %d out of range", f, a);
    if (b >= 0) {
      if (b >= nc) return ctx.fail(FV3D_ERR_BOUNDS, "face %d: cell %d out of range", f, b);
      if (b == a) return ctx.fail(FV3D_ERR_INVALID_ARG, "face %d joins cell %d to itself", f, a);
      if (bf >= 0) return ctx.fail(FV3D_ERR_INVALID_ARG, "interior face %d has boundary %d", f, bf);
    } else {
      if (b != -1 || bf < 0 || bf >= nb)
        return ctx.fail(FV3D_ERR_BOUNDS, "face %d: bad boundary index %d", f, bf);
      if (m.boundary_face[bf] != f)
        return ctx.fail(FV3D_ERR_INVALID_ARG, "boundary %d does not point back to face %d", bf, f);
      ++n_bfaces;
    }
    if (!(m.face_area[f] > 0.0) || !(m.face_lambda[f] > 0.0) || !(m.face_lambda[f] <= 1.0))
      return ctx.fail(FV3D_ERR_INVALID_ARG, "face %d: bad area or weight", f);
  }
  if (n_bfaces != nb) return ctx.fail(FV3D_ERR_INVALID_ARG, "%d boundary faces but %d boundaries", n_bfaces, nb);
  for (int b = 0; b < nb; ++b) {
    int r = m.boundary_id[b];
    if (r < 0 || r >= m.n_regions || m.region_is_boundary[r] == 0)
      return ctx.fail(FV3D_ERR_BOUNDS, "boundary %d: bad region %d", b, r);
  }
  // cell face lists from the faces, ascending reference face id: the order
  // in which the reference's face scatter (finite_volume.c:100-111) and
  // Green-Gauss loop (reconstruction.c:43-71) accumulate into a cell
  std::vector<int> cnt(nc, 0);
  for (int f = 0; f < nf; ++f) {
    cnt[m.face_cells[2 * f]]++;
    if (m.face_cells[2 * f + 1] >= 0) cnt[m.face_cells[2 * f + 1]]++;
  }
  for (int i = 0; i < nc; ++i) {
    if (cnt[i] != m.cell_n_faces[i] || cnt[i] > mcf)
      return ctx.fail(FV3D_ERR_INVALID_ARG, "cell %d: %d faces reference it, n_faces says %d", i, cnt[i],
                      m.cell_n_faces[i]);
    for (int k = 0; k < m.cell_n_faces[i]; ++k) {
      int f = m.cell_faces[(size_t)i * mcf + k];
      if (f < 0 || f >= nf) return ctx.fail(FV3D_ERR_BOUNDS, "cell %d: face %d out of range", i, f);
      if (m.face_cells[2 * f] != i && m.face_cells[2 * f + 1] != i)
        return ctx.fail(FV3D_ERR_INVALID_ARG, "cell %d lists face %d that does not touch it", i, f);
    }
  }

  // ---- renumbering ----
  std::vector<int> order;
  if (ctx.cfg.renumber == FV3D_RENUMBER_MORTON) {
    order = morton_order(nc, m.cell_x);
  } else if (ctx.cfg.renumber == FV3D_RENUMBER_RCM) {
    std::vector<std::vector<int>> adj(nc);
    for (int f = 0; f < nf; ++f) {
      int a = m.face_cells[2 * f], b = m.face_cells[2 * f + 1];
      if (b >= 0) { adj[a].push_back(b); adj[b].push_back(a); }
    }
    order = rcm_order(nc, adj);
  } else {
    order.resize(nc);
    std::iota(order.begin(), order.end(), 0);
  }
  ctx.perm = order;
  ctx.iperm.assign(nc, 0);
  for (int i = 0; i < nc; ++i) ctx.iperm[order[i]] = i;

  // face order: interior faces by (min new cell, max new cell, id), then
  // boundary faces by (new cell, id); orientation (cell 0 / cell 1) kept
  std::vector<int> faces(nf);
  std::iota(faces.begin(), faces.end(), 0);
  auto key = [&](int f) {
    int a = ctx.iperm[m.face_cells[2 * f]];
    int b = m.face_cells[2 * f + 1];
    if (b < 0) return std::make_tuple(1, a, 0, f);
    b = ctx.iperm[b];
    return std::make_tuple(0, std::min(a, b), std::max(a, b), f);
  };
  std::sort(faces.begin(), faces.end(), [&](int x, int y) { return key(x) < key(y); });
  ctx.fperm = faces;
  std::vector<int> ifperm(nf);
  for (int i = 0; i < nf; ++i) ifperm[faces[i]] = i;
  ctx.nc = nc; ctx.nf = nf; ctx.nb = nb; ctx.mcf = mcf; ctx.nf_int = nf - nb; ctx.n_regions = m.n_regions;

  // ---- metrics (mesh.c:19-83) and per-face arrays in the new order ----
  ctx.h_fc0.assign(nf, 0);
  ctx.h_fc1.assign(nf, 0);
  ctx.h_fregion.assign(nb, 0);
  ctx.h_geo.assign((size_t)nf * GEO, 0.0);
  ctx.h_lam.assign(nf, 0.0);
  std::vector<double> d1((size_t)nf * 3), d2((size_t)nf * 3);
  for (int nfid = 0; nfid < nf; ++nfid) {
    const int f = faces[nfid];
    const int a = m.face_cells[2 * f], b = m.face_cells[2 * f + 1];
    ctx.h_fc0[nfid] = ctx.iperm[a];
    double* g = &ctx.h_geo[(size_t)nfid * GEO];
    for (int d = 0; d < 3; ++d) {
      g[G_N + d] = m.face_n[3 * f + d];
      g[G_T1 + d] = m.face_t1[3 * f + d];
      g[G_T2 + d] = m.face_t2[3 * f + d];
      g[G_D1 + d] = m.face_x[3 * f + d] - m.cell_x[3 * a + d];
      g[G_D2 + d] = 0.0;
    }
    g[G_A] = m.face_area[f];
    ctx.h_lam[nfid] = m.face_lambda[f];
    if (b >= 0) {
      ctx.h_fc1[nfid] = ctx.iperm[b];
      for (int d = 0; d < 3; ++d)
        g[G_D2 + d] = m.face_dist_cell_2 ? m.face_dist_cell_2[3 * f + d]
                                         : m.face_x[3 * f + d] - m.cell_x[3 * b + d];
    } else {
      const int bidx = m.face_boundary[f];
      ctx.h_fc1[nfid] = nc + (nfid - ctx.nf_int);  // ghost index
      ctx.h_fregion[nfid - ctx.nf_int] = m.boundary_id[bidx];
    }
    for (int d = 0; d < 3; ++d) {
      d1[3 * (size_t)nfid + d] = g[G_D1 + d];
      d2[3 * (size_t)nfid + d] = g[G_D2 + d];
    }
  }
  // cell face lists: entries (new face << 1) | side, ascending reference id;
  // the stride is padded to 4, 6 or 8 (the face-count variants the kernels
  // are compiled for)
  const int mcf_pad = (mcf <= 4) ? 4 : (mcf <= 6 ? 6 : 8);
  ctx.mcf = mcf_pad;
  ctx.h_cface.assign((size_t)nc * mcf_pad, -1);
  ctx.h_vol.assign(nc, 0.0);
  ctx.h_dx.assign((size_t)nc * 3, 0.0);
  ctx.vol_total = 0.0;
  for (int i = 0; i < nc; ++i) ctx.vol_total += m.cell_volume[i];  // sum_n order (mesh.c:25)
  ctx.h_cell_x.assign(m.cell_x, m.cell_x + (size_t)nc * 3);
  for (int c = 0; c < nc; ++c) {
    const int old = order[c];
    std::vector<int> fl;
    for (int k = 0; k < m.cell_n_faces[old]; ++k) fl.push_back(m.cell_faces[(size_t)old * mcf + k]);
    std::sort(fl.begin(), fl.end());
    for (size_t k = 0; k < fl.size(); ++k) {
      const int f = fl[k];
      const int side = (m.face_cells[2 * f] == old) ? 0 : 1;
      ctx.h_cface[(size_t)c * mcf_pad + k] = (ifperm[f] << 1) | side;
    }
    ctx.h_vol[c] = m.cell_volume[old];
    for (int d = 0; d < 3; ++d) ctx.h_dx[3 * (size_t)c + d] = m.cell_dx[3 * old + d];
  }
  // least-squares weights w = M^-1 d per face side (unweighted LSQ; for a
  // boundary face d = x_f - x_c with the ghost value)
  ctx.h_lsq.assign((size_t)nf * 6, 0.0);
  if (ctx.cfg.gradient == FV3D_GRADIENT_LEAST_SQUARES) {
    for (int c = 0; c < nc; ++c) {
      double M[6] = {0, 0, 0, 0, 0, 0};
      double dv[8][3];
      int nfc = 0;
      for (int k = 0; k < mcf_pad; ++k) {
        int e = ctx.h_cface[(size_t)c * mcf_pad + k];
        if (e < 0) break;
        int f = e >> 1, side = e & 1;
        for (int q = 0; q < 3; ++q) {
          if (side == 0)
            dv[k][q] = (f >= ctx.nf_int) ? d1[3 * (size_t)f + q] : d1[3 * (size_t)f + q] - d2[3 * (size_t)f + q];
          else
            dv[k][q] = d2[3 * (size_t)f + q] - d1[3 * (size_t)f + q];
        }
        M[0] += dv[k][0] * dv[k][0];
        M[1] += dv[k][0] * dv[k][1];
        M[2] += dv[k][0] * dv[k][2];
        M[3] += dv[k][1] * dv[k][1];
        M[4] += dv[k][1] * dv[k][2];
        M[5] += dv[k][2] * dv[k][2];
        nfc = k + 1;
      }
      double c00 = M[3] * M[5] - M[4] * M[4];
      double c01 = M[2] * M[4] - M[1] * M[5];
      double c02 = M[1] * M[4] - M[2] * M[3];
      double c11 = M[0] * M[5] - M[2] * M[2];
      double c12 = M[1] * M[2] - M[0] * M[4];
      double c22 = M[0] * M[3] - M[1] * M[1];
      double det = M[0] * c00 + M[1] * c01 + M[2] * c02;
      if (!(std::fabs(det) > 0.0)) return ctx.fail(FV3D_ERR_INVALID_ARG, "cell %d: singular least-squares matrix", order[c]);
      double s = 1.0 / det;
      for (int k = 0; k < nfc; ++k) {
        int e = ctx.h_cface[(size_t)c * mcf_pad + k];
        int f = e >> 1, side = e & 1;
        double* w = &ctx.h_lsq[6 * (size_t)f + 3 * side];
        w[0] = s * (c00 * dv[k][0] + c01 * dv[k][1] + c02 * dv[k][2]);
        w[1] = s * (c01 * dv[k][0] + c11 * dv[k][1] + c12 * dv[k][2]);
        w[2] = s * (c02 * dv[k][0] + c12 * dv[k][1] + c22 * dv[k][2]);
      }
    }
  }
  return FV3D_OK;
}

#define UP(buf, src, count)                                                                   \
  do {                                                                                        \
    cudaError_t e__ = (buf).alloc(count);                                                     \
    if (e__ == cudaSuccess)                                                                   \
      e__ = cudaMemcpy((buf).p, (src), sizeof(*(buf).p) * (count), cudaMemcpyHostToDevice);   \
    if (e__ != cudaSuccess) return ctx.cuda(e__, "mesh upload");                              \
  } while (0)

#define ALLOC(buf, count)                                                                     \
  do {                                                                                        \
    cudaError_t e__ = (buf).alloc(count);                                                     \
    if (e__ == cudaSuccess) e__ = cudaMemset((buf).p, 0, sizeof(*(buf).p) * (count));         \
    if (e__ != cudaSuccess) return ctx.cuda(e__, "device allocation");                        \
  } while (0)

// Data every path needs; the FP64-path and mixed-path arrays follow in
// ensure_fp64_path / ensure_mixed_path (the explicit path allocates the one
// of its precision, the implicit solver both).
fv3d_status upload_mesh(Ctx& ctx) {
  ctx.free_device();
  const int nc = ctx.nc, nf = ctx.nf;
  ctx.ncp = (nc + kTile - 1) / kTile * kTile;
  UP(ctx.d_perm, ctx.perm.data(), (size_t)nc);
  UP(ctx.d_iperm, ctx.iperm.data(), (size_t)nc);
  UP(ctx.d_fc0, ctx.h_fc0.data(), (size_t)nf);
  UP(ctx.d_fc1, ctx.h_fc1.data(), (size_t)nf);
  if (ctx.nb > 0) UP(ctx.d_fregion, ctx.h_fregion.data(), (size_t)ctx.nb);
  {
    // ctx.mcf = padded stride; rows up to ncp (whole tiles for the staged gradient pass)
    std::vector<int> cf((size_t)ctx.ncp * ctx.mcf, -1);
    std::copy(ctx.h_cface.begin(), ctx.h_cface.end(), cf.begin());
    UP(ctx.d_cface, cf.data(), cf.size());
  }
  UP(ctx.d_vol, ctx.h_vol.data(), (size_t)nc);
  UP(ctx.d_dx, ctx.h_dx.data(), (size_t)nc * 3);
  ALLOC(ctx.d_U, (size_t)nc * 5);
  ALLOC(ctx.d_dphi, (size_t)nc * 5);
  ALLOC(ctx.d_stage, (size_t)nc * 10);
  ALLOC(ctx.d_part, (size_t)((nc + 255) / 256 + 1) * 5 + 5);
  ALLOC(ctx.d_sc, 1);
  ALLOC(ctx.d_bits, 2);
  ctx.mesh_ready = true;
  fv3d_status st = ctx.fp64() ? ensure_fp64_path(ctx) : ensure_mixed_path(ctx);
  if (st != FV3D_OK) ctx.mesh_ready = false;
  return st;
}

fv3d_status ensure_fp64_path(Ctx& ctx) {
  if (ctx.d_rec.p != nullptr) return FV3D_OK;
  const int nc = ctx.nc, nf = ctx.nf;
  std::vector<double> rvol(nc);
  for (int i = 0; i < nc; ++i) rvol[i] = 1.0 / ctx.h_vol[i];  // s_volume (reconstruction.c:82)
  auto up_d = [&](DevBuf<char>& b, const std::vector<double>& src) -> fv3d_status {
    cudaError_t e = b.alloc(src.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(b.p, src.data(), src.size() * sizeof(double), cudaMemcpyHostToDevice);
    return ctx.cuda(e, "mesh upload");
  };
  fv3d_status st;
  if ((st = up_d(ctx.d_geo, ctx.h_geo)) != FV3D_OK) return st;
  if ((st = up_d(ctx.d_lam, ctx.h_lam)) != FV3D_OK) return st;
  if ((st = up_d(ctx.d_lsq, ctx.h_lsq)) != FV3D_OK) return st;
  if ((st = up_d(ctx.d_rvol, rvol)) != FV3D_OK) return st;
  ALLOC(ctx.d_K, (size_t)nc * 5);
  ALLOC(ctx.d_U0, (size_t)nc * 5);
  ALLOC(ctx.d_FA, (size_t)nf * FAS * sizeof(double));
  ALLOC(ctx.d_rec, (size_t)nc * REC * sizeof(double));
  ALLOC(ctx.d_Pq, (size_t)nc * 5);
  return FV3D_OK;
}

fv3d_status ensure_mixed_path(Ctx& ctx) {
  if (ctx.d_fs.p != nullptr) return FV3D_OK;
  const int nc = ctx.nc, nf = ctx.nf;
  // per (cell, face slot) geometry, read coalesced by the cell kernels:
  // face (n, A) in its cell 0 -> cell 1 orientation, this side's d with the
  // Green-Gauss weight (lambda on the cell-0 side, 1 - lambda on the cell-1
  // side), this side's least-squares weights
  const int mcf = ctx.mcf;
  std::vector<int2> fcell(nf);
  for (int f = 0; f < nf; ++f) fcell[f] = make_int2(ctx.h_fc0[f], ctx.h_fc1[f]);
  std::vector<float4> sN((size_t)nc * mcf, make_float4(0.f, 0.f, 0.f, 0.f)), sD(sN), sW(sN);
  for (int c = 0; c < nc; ++c)
    for (int k = 0; k < mcf; ++k) {
      const int e = ctx.h_cface[(size_t)c * mcf + k];
      if (e < 0) break;
      const int f = e >> 1, side = e & 1;
      const double* g = &ctx.h_geo[(size_t)f * GEO];
      const size_t i = (size_t)c * mcf + k;
      sN[i] = make_float4((float)g[G_N], (float)g[G_N + 1], (float)g[G_N + 2], (float)g[G_A]);
      const double* d = side ? &g[G_D2] : &g[G_D1];
      const double w = side ? 1.0 - ctx.h_lam[f] : ctx.h_lam[f];
      sD[i] = make_float4((float)d[0], (float)d[1], (float)d[2], (float)w);
      const double* lw = &ctx.h_lsq[6 * (size_t)f + 3 * side];
      sW[i] = make_float4((float)lw[0], (float)lw[1], (float)lw[2], 0.f);
    }
  // per cell: sum_f s_f n_f A_f (closure of the Green-Gauss difference
  // form) with 1/V, and (dx, V) for the time step
  std::vector<float4> cg(ctx.ncp, make_float4(0.f, 0.f, 0.f, 0.f)), cd(cg);
  for (int c = 0; c < nc; ++c) {
    double S[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < ctx.mcf; ++k) {
      const int e = ctx.h_cface[(size_t)c * ctx.mcf + k];
      if (e < 0) break;
      const double* g = &ctx.h_geo[(size_t)(e >> 1) * GEO];
      const double sg = (e & 1) ? -g[G_A] : g[G_A];
      for (int d = 0; d < 3; ++d) S[d] += sg * g[G_N + d];
    }
    cg[c] = make_float4((float)S[0], (float)S[1], (float)S[2], (float)(1.0 / ctx.h_vol[c]));
    cd[c] = make_float4((float)ctx.h_dx[3 * (size_t)c], (float)ctx.h_dx[3 * (size_t)c + 1],
                        (float)ctx.h_dx[3 * (size_t)c + 2], (float)ctx.h_vol[c]);
  }
  // neighbour of every face slot: cell, -1 for a ghost, -2 for padding
  std::vector<int> nbr((size_t)ctx.ncp * ctx.mcf, -2);
  for (int c = 0; c < nc; ++c)
    for (int k = 0; k < ctx.mcf; ++k) {
      const int e = ctx.h_cface[(size_t)c * ctx.mcf + k];
      if (e < 0) break;
      const int f = e >> 1;
      nbr[(size_t)c * ctx.mcf + k] = (f >= ctx.nf_int) ? -1 : ((e & 1) ? ctx.h_fc0[f] : ctx.h_fc1[f]);
    }
  // the record of each slot's other side: the neighbour's own side in the
  // slot that lists the same face, or the ghost side of a boundary face
  std::vector<int> oth((size_t)ctx.ncp * ctx.mcf, -1);
  for (int c = 0; c < nc; ++c)
    for (int k = 0; k < ctx.mcf; ++k) {
      const int e = ctx.h_cface[(size_t)c * ctx.mcf + k];
      if (e < 0) break;
      const int f = e >> 1, side = e & 1;
      long long idx;
      if (f >= ctx.nf_int) {
        idx = (long long)ctx.mcf * ctx.ncp + (f - ctx.nf_int);
      } else {
        const int n = side ? ctx.h_fc0[f] : ctx.h_fc1[f];
        int kn = -1;
        for (int j = 0; j < ctx.mcf; ++j) {
          const int en = ctx.h_cface[(size_t)n * ctx.mcf + j];
          if (en < 0) break;
          if ((en >> 1) == f) { kn = j; break; }
        }
        if (kn < 0) return ctx.fail(FV3D_ERR_INVALID_ARG, "face %d missing from its cell %d", f, n);
        idx = (long long)kn * ctx.ncp + n;
      }
      oth[(size_t)c * ctx.mcf + k] = (int)((idx << 1) | side);
    }
  UP(ctx.d_cgeo, cg.data(), cg.size());
  UP(ctx.d_cdx, cd.data(), cd.size());
  UP(ctx.d_cnbr, nbr.data(), nbr.size());
  UP(ctx.d_cother, oth.data(), oth.size());
  UP(ctx.d_fcell, fcell.data(), (size_t)nf);
  UP(ctx.d_slotN, sN.data(), sN.size());
  UP(ctx.d_slotD, sD.data(), sD.size());
  // slot-major copies [mcf][ncp] (rows padded to whole tiles with zeros):
  // the flux pass reads slotNk, the staged gradient pass copies one row
  // segment per slot into shared memory
  auto slot_major = [&](const std::vector<float4>& src, DevBuf<float4>& dst) -> fv3d_status {
    std::vector<float4> t((size_t)mcf * ctx.ncp, make_float4(0.f, 0.f, 0.f, 0.f));
    for (int c = 0; c < nc; ++c)
      for (int k = 0; k < mcf; ++k) t[(size_t)k * ctx.ncp + c] = src[(size_t)c * mcf + k];
    UP(dst, t.data(), t.size());
    return FV3D_OK;
  };
  fv3d_status st;
  if ((st = slot_major(sN, ctx.d_slotNk)) != FV3D_OK) return st;
  if ((st = slot_major(sD, ctx.d_slotDk)) != FV3D_OK) return st;
  if (ctx.cfg.gradient == FV3D_GRADIENT_LEAST_SQUARES) {
    UP(ctx.d_slotW, sW.data(), sW.size());
    if ((st = slot_major(sW, ctx.d_slotWk)) != FV3D_OK) return st;
  }
  {
    cudaError_t e = setup_mx_sides();
    if (e != cudaSuccess) return ctx.cuda(e, "gradient-pass setup");
  }
  ALLOC(ctx.d_Uf, (size_t)ctx.ncp * 8);
  ALLOC(ctx.d_UfN, (size_t)ctx.ncp * 8);
  ALLOC(ctx.d_kf, (size_t)ctx.ncp * 5);
  ALLOC(ctx.d_dU, (size_t)ctx.ncp * 5);
  // face-side records: every cell's own sides slot-major, then the ghost sides
  const size_t nrec = (size_t)ctx.mcf * ctx.ncp + (size_t)(nf - ctx.nf_int);
  ALLOC(ctx.d_fs, nrec * 8);
  ALLOC(ctx.d_fsv, nrec);
  return FV3D_OK;
}

}  // namespace fv3d
