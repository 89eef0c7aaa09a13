// ls_layout.cpp -- host construction of the patch layout (setup, not the
// time step).  All orderings are stable counting sorts, so the result is
// deterministic and equal to the reference's thrust stable radix sorts:
//   copies by patch      src/core3d/cuda/meshFIM3d.cu:461-469 (K3 + sort_by_key)
//   vertices by patch    src/core3d/cuda/meshFIM3d.cu:503-511
//   slots by vertex      src/core3d/cuda/meshFIM3d.cu:537-542
//   patch adjacency      src/core3d/cuda/meshFIM3d.cu:546-570
#include "ls_layout.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace lsgb {

void tet_local_coords(const float P[4][3], float Lc[6]) {
  float AB[3] = {P[1][0] - P[0][0], P[1][1] - P[0][1], P[1][2] - P[0][2]};
  float AC[3] = {P[2][0] - P[0][0], P[2][1] - P[0][1], P[2][2] - P[0][2]};
  float AD[3] = {P[3][0] - P[0][0], P[3][1] - P[0][1], P[3][2] - P[0][2]};
  float lenAB = std::sqrt(AB[0] * AB[0] + AB[1] * AB[1] + AB[2] * AB[2]);
  float N[3] = {AB[1] * AC[2] - AB[2] * AC[1], AB[2] * AC[0] - AB[0] * AC[2],
                AB[0] * AC[1] - AB[1] * AC[0]};
  float lenN = std::sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
  float Z[3] = {N[0] / lenN, N[1] / lenN, N[2] / lenN};
  float X[3] = {AB[0] / lenAB, AB[1] / lenAB, AB[2] / lenAB};
  float Y[3] = {Z[1] * X[2] - Z[2] * X[1], Z[2] * X[0] - Z[0] * X[2], Z[0] * X[1] - Z[1] * X[0]};
  Lc[0] = lenAB;
  Lc[1] = AC[0] * X[0] + AC[1] * X[1] + AC[2] * X[2];
  Lc[2] = AC[0] * Y[0] + AC[1] * Y[1] + AC[2] * Y[2];
  Lc[3] = AD[0] * X[0] + AD[1] * X[1] + AD[2] * X[2];
  Lc[4] = AD[0] * Y[0] + AD[1] * Y[1] + AD[2] * Y[2];
  Lc[5] = AD[0] * Z[0] + AD[1] * Z[1] + AD[2] * Z[2];
}

void tri_local_coords(const double P[3][3], const double vel[3], double Lc[3], double sig[2]) {
  double AB[3] = {P[1][0] - P[0][0], P[1][1] - P[0][1], P[1][2] - P[0][2]};
  double AC[3] = {P[2][0] - P[0][0], P[2][1] - P[0][1], P[2][2] - P[0][2]};
  double cr[3] = {AB[1] * AC[2] - AB[2] * AC[1], AB[2] * AC[0] - AB[0] * AC[2],
                  AB[0] * AC[1] - AB[1] * AC[0]};
  double Y[3] = {cr[1] * AB[2] - cr[2] * AB[1], cr[2] * AB[0] - cr[0] * AB[2],
                 cr[0] * AB[1] - cr[1] * AB[0]};
  double lenY = std::sqrt(Y[0] * Y[0] + Y[1] * Y[1] + Y[2] * Y[2]);
  double lenAB = std::sqrt(AB[0] * AB[0] + AB[1] * AB[1] + AB[2] * AB[2]);
  Lc[0] = lenAB;
  Lc[1] = (AC[0] * AB[0] + AC[1] * AB[1] + AC[2] * AB[2]) / lenAB;
  Lc[2] = (AC[0] * Y[0] + AC[1] * Y[1] + AC[2] * Y[2]) / lenY;
  sig[0] = (vel[0] * AB[0] + vel[1] * AB[1] + vel[2] * AB[2]) / lenAB;
  sig[1] = (vel[0] * Y[0] + vel[1] * Y[1] + vel[2] * Y[2]) / lenY;
}

std::string build_layout(int dim, int nv, const float* xyz, int ne, const int* elems,
                         const int* npart, int nparts, Layout& L) {
  if (dim != 2 && dim != 3) return "dimension must be 2 or 3";
  if (nv <= 0 || ne <= 0 || nparts <= 0) return "empty mesh or partition";
  const int d1 = dim + 1;
  for (int v = 0; v < nv; ++v)
    if (npart[v] < 0 || npart[v] >= nparts) return "partition label out of range";
  for (long long i = 0; i < (long long)ne * d1; ++i)
    if (elems[i] < 0 || elems[i] >= nv) return "element vertex index out of range";
  L = Layout();
  L.dim = dim; L.nv = nv; L.ne = ne; L.nparts = nparts;

  // distinct patches of each element in vertex order (K2/K3)
  auto distinct = [&](int e, int* parts) {
    const int* ev = elems + (size_t)e * d1;
    int n = 0;
    for (int k = 0; k < d1; ++k) {
      int pk = npart[ev[k]];
      bool dup = false;
      for (int j = 0; j < n; ++j) dup |= (parts[j] == pk);
      if (!dup) parts[n++] = pk;
    }
    return n;
  };
  std::vector<long long> pcnt(nparts + 1, 0);
  long long full = 0;
  for (int e = 0; e < ne; ++e) {
    int parts[4];
    int n = distinct(e, parts);
    for (int j = 0; j < n; ++j) pcnt[parts[j] + 1]++;
    full += n;
  }
  if (full >= INT_MAX / 4) return "too many element copies";
  L.full = full;
  L.ele_offsets.assign(nparts + 1, 0);
  for (int p = 0; p < nparts; ++p) {
    L.ele_offsets[p + 1] = (int)(L.ele_offsets[p] + pcnt[p + 1]);
    L.lep = std::max<int>(L.lep, (int)pcnt[p + 1]);
  }
  L.ele_permute.resize(full);
  {
    std::vector<int> f(L.ele_offsets.begin(), L.ele_offsets.end() - 1);
    for (int e = 0; e < ne; ++e) {
      int parts[4];
      int n = distinct(e, parts);
      for (int j = 0; j < n; ++j) L.ele_permute[f[parts[j]]++] = e;
    }
  }
  // vertices by patch (stable)
  std::vector<int> vcnt(nparts + 1, 0);
  for (int v = 0; v < nv; ++v) vcnt[npart[v] + 1]++;
  L.vert_offsets.assign(nparts + 1, 0);
  for (int p = 0; p < nparts; ++p) {
    if (vcnt[p + 1] == 0) return "a patch has no vertices";
    if (pcnt[p + 1] == 0) return "a patch has no elements";
    L.vert_offsets[p + 1] = L.vert_offsets[p] + vcnt[p + 1];
    L.lvp = std::max(L.lvp, vcnt[p + 1]);
  }
  L.vert_permute.resize(nv);
  L.vert_ipermute.resize(nv);
  {
    std::vector<int> f(L.vert_offsets.begin(), L.vert_offsets.end() - 1);
    for (int v = 0; v < nv; ++v) {
      int n = f[npart[v]]++;
      L.vert_permute[n] = v;
      L.vert_ipermute[v] = n;
    }
  }
  std::vector<int> vpart(nv);
  for (int p = 0; p < nparts; ++p)
    for (int v = L.vert_offsets[p]; v < L.vert_offsets[p + 1]; ++v) vpart[v] = p;
  // copy connectivity in new ids
  L.conn.resize((size_t)full * d1);
  for (long long c = 0; c < full; ++c) {
    const int* ev = elems + (size_t)L.ele_permute[c] * d1;
    for (int k = 0; k < d1; ++k) L.conn[c * d1 + k] = L.vert_ipermute[ev[k]];
  }
  L.xyz_p.resize((size_t)3 * nv);
  for (int v = 0; v < nv; ++v)
    for (int j = 0; j < 3; ++j) L.xyz_p[(size_t)j * nv + v] = xyz[(size_t)L.vert_permute[v] * 3 + j];
  // LIM and mean edge length
  {
    std::vector<int> adj(nv, 0);
    double esum = 0;
    long long ecount = 0;
    for (int e = 0; e < ne; ++e) {
      const int* ev = elems + (size_t)e * d1;
      for (int k = 0; k < d1; ++k) adj[ev[k]]++;
      for (int a = 0; a < d1; ++a)
        for (int b = a + 1; b < d1; ++b) {
          double dx = (double)xyz[(size_t)ev[a] * 3] - xyz[(size_t)ev[b] * 3];
          double dy = (double)xyz[(size_t)ev[a] * 3 + 1] - xyz[(size_t)ev[b] * 3 + 1];
          double dz = (double)xyz[(size_t)ev[a] * 3 + 2] - xyz[(size_t)ev[b] * 3 + 2];
          esum += std::sqrt(dx * dx + dy * dy + dz * dz);
          ecount++;
        }
    }
    L.lim = *std::max_element(adj.begin(), adj.end());
    L.mean_edge = esum / (double)ecount;
  }
  // ghosts per patch and slab-local connectivity
  L.ghost_offsets.assign(nparts + 1, 0);
  L.conn_local.assign((size_t)full * 4, 0xffff);
  {
    std::vector<int> mark(nv, -1), gl;
    std::vector<int> local(nv, 0);
    for (int p = 0; p < nparts; ++p) {
      gl.clear();
      const int vs = L.vert_offsets[p];
      for (int c = L.ele_offsets[p]; c < L.ele_offsets[p + 1]; ++c)
        for (int k = 0; k < d1; ++k) {
          int v = L.conn[(size_t)c * d1 + k];
          if (vpart[v] != p && mark[v] != p) { mark[v] = p; gl.push_back(v); }
        }
      std::sort(gl.begin(), gl.end());
      const int nvp = L.vert_offsets[p + 1] - vs;
      if (nvp + (int)gl.size() >= 0xffff) return "patch slab exceeds 65535 vertices";
      for (size_t j = 0; j < gl.size(); ++j) local[gl[j]] = nvp + (int)j;
      for (int c = L.ele_offsets[p]; c < L.ele_offsets[p + 1]; ++c)
        for (int k = 0; k < d1; ++k) {
          int v = L.conn[(size_t)c * d1 + k];
          L.conn_local[(size_t)c * 4 + k] = (uint16_t)(vpart[v] == p ? v - vs : local[v]);
        }
      L.ghost_offsets[p + 1] = L.ghost_offsets[p] + (int)gl.size();
      L.ghost_ids.insert(L.ghost_ids.end(), gl.begin(), gl.end());
      L.lgp = std::max(L.lgp, (int)gl.size());
    }
  }
  // owned-vertex slot lists (k-major, then copy order)
  {
    std::vector<int> cpart(full);
    for (int p = 0; p < nparts; ++p)
      for (int c = L.ele_offsets[p]; c < L.ele_offsets[p + 1]; ++c) cpart[c] = p;
    L.vslot_off.assign((size_t)nv + 1, 0);
    for (int k = 0; k < d1; ++k)
      for (long long c = 0; c < full; ++c) {
        int v = L.conn[c * d1 + k];
        if (cpart[c] == vpart[v]) L.vslot_off[v + 1]++;
      }
    for (int v = 0; v < nv; ++v) {
      if (L.vslot_off[v + 1] == 0) return "a vertex belongs to no element";
      L.vslot_off[v + 1] += L.vslot_off[v];
    }
    L.vslot.resize(L.vslot_off[nv]);
    std::vector<int> f(L.vslot_off.begin(), L.vslot_off.end() - 1);
    for (int k = 0; k < d1; ++k)
      for (long long c = 0; c < full; ++c) {
        int v = L.conn[c * d1 + k];
        int p = cpart[c];
        if (p == vpart[v]) L.vslot[f[v]++] = (uint16_t)((c - L.ele_offsets[p]) * 4 + k);
      }
    if (L.lep * 4 > 0xffff) return "patch has too many element copies";
    // corners beyond the reference's per-vertex slot limit
    const int cap = ref_slot_cap(dim);
    L.slot_capped.assign(full, 0);
    L.any_capped = false;
    for (int v = 0; v < nv; ++v)
      for (int q = L.vslot_off[v] + cap; q < L.vslot_off[v + 1]; ++q) {
        const int sl = L.vslot[q];
        L.slot_capped[L.ele_offsets[vpart[v]] + (sl >> 2)] |= (uint8_t)(1u << (sl & 3));
        L.any_capped = true;
      }
  }
  // patch adjacency: every copy of p holds a vertex of p, so the patches of
  // its other vertices are exactly those joined to p by a mesh edge
  {
    std::vector<int> mark(nparts, -1);
    L.padj_off.assign(nparts + 1, 0);
    for (int p = 0; p < nparts; ++p) {
      size_t s0 = L.padj.size();
      for (int c = L.ele_offsets[p]; c < L.ele_offsets[p + 1]; ++c) {
        int own = 0;
        for (int k = 0; k < d1; ++k) {
          int q = vpart[L.conn[(size_t)c * d1 + k]];
          if (q == p) own++;
          else if (mark[q] != p) { mark[q] = p; L.padj.push_back(q); }
        }
        if (own >= 2) L.has_internal_edge = true;
      }
      std::sort(L.padj.begin() + s0, L.padj.end());
      L.padj_off[p + 1] = (int)L.padj.size();
    }
  }
  return "";
}

std::string merge_layouts(const std::vector<const Layout*>& parts, Layout& out) {
  out = Layout();
  if (parts.empty()) return "no meshes";
  const int dim = parts[0]->dim;
  long long nv = 0, ne = 0, np = 0, full = 0, ng = 0, ns = 0, na = 0;
  for (const Layout* P : parts) {
    if (P->dim != dim) return "meshes of different dimension";
    nv += P->nv; ne += P->ne; np += P->nparts; full += P->full;
    ng += (long long)P->ghost_ids.size(); ns += (long long)P->vslot.size(); na += (long long)P->padj.size();
  }
  if (nv > INT32_MAX || ne > INT32_MAX || np > INT32_MAX || full > INT32_MAX || ng > INT32_MAX || ns > INT32_MAX ||
      na > INT32_MAX)
    return "batch too large for 32-bit indices";
  out.dim = dim;
  out.nv = (int)nv; out.ne = (int)ne; out.nparts = (int)np; out.full = full;
  const int d1 = dim + 1;
  out.vert_permute.reserve(nv); out.vert_ipermute.reserve(nv);
  out.vert_offsets.reserve(np + 1); out.ele_offsets.reserve(np + 1);
  out.ghost_offsets.reserve(np + 1); out.padj_off.reserve(np + 1);
  out.vslot_off.reserve(nv + 1);
  out.ele_permute.reserve(full); out.conn.reserve(full * d1); out.conn_local.reserve(full * 4);
  out.ghost_ids.reserve(ng); out.vslot.reserve(ns); out.padj.reserve(na);
  out.slot_capped.reserve(full);
  out.xyz_p.assign((size_t)nv * 3, 0.f);
  out.patch_mesh.reserve(np);
  out.vert_offsets.push_back(0); out.ele_offsets.push_back(0); out.ghost_offsets.push_back(0);
  out.padj_off.push_back(0); out.vslot_off.push_back(0);
  int vb = 0, eb = 0, pb = 0, cb = 0, gb = 0, sb = 0, ab = 0;
  for (size_t k = 0; k < parts.size(); ++k) {
    const Layout& P = *parts[k];
    for (int v = 0; v < P.nv; ++v) {
      out.vert_permute.push_back(vb + P.vert_permute[v]);
      out.vert_ipermute.push_back(vb + P.vert_ipermute[v]);
      out.vslot_off.push_back(sb + P.vslot_off[v + 1]);
      for (int j = 0; j < 3; ++j) out.xyz_p[(size_t)j * nv + vb + v] = P.xyz_p[(size_t)j * P.nv + v];
    }
    for (int p = 0; p < P.nparts; ++p) {
      out.vert_offsets.push_back(vb + P.vert_offsets[p + 1]);
      out.ele_offsets.push_back(cb + P.ele_offsets[p + 1]);
      out.ghost_offsets.push_back(gb + P.ghost_offsets[p + 1]);
      out.padj_off.push_back(ab + P.padj_off[p + 1]);
      out.patch_mesh.push_back((int)k);
    }
    for (long long c = 0; c < P.full; ++c) out.ele_permute.push_back(eb + P.ele_permute[c]);
    for (int x : P.conn) out.conn.push_back(vb + x);
    out.conn_local.insert(out.conn_local.end(), P.conn_local.begin(), P.conn_local.end());
    for (int g : P.ghost_ids) out.ghost_ids.push_back(vb + g);
    out.vslot.insert(out.vslot.end(), P.vslot.begin(), P.vslot.end());
    out.slot_capped.insert(out.slot_capped.end(), P.slot_capped.begin(), P.slot_capped.end());
    out.any_capped = out.any_capped || P.any_capped;
    for (int q : P.padj) out.padj.push_back(pb + q);
    out.lep = std::max(out.lep, P.lep);
    out.lvp = std::max(out.lvp, P.lvp);
    out.lgp = std::max(out.lgp, P.lgp);
    out.lim = std::max(out.lim, P.lim);
    out.has_internal_edge = out.has_internal_edge || P.has_internal_edge;
    out.mesh_edge.push_back(P.mean_edge);
    vb += P.nv; eb += P.ne; pb += P.nparts; cb += (int)P.full;
    gb += (int)P.ghost_ids.size(); sb += (int)P.vslot.size(); ab += (int)P.padj.size();
  }
  // the union's mean edge (used only where one FIM frame serves all meshes)
  double w = 0, s = 0;
  for (const Layout* P : parts) { w += (double)P->ne; s += P->mean_edge * (double)P->ne; }
  out.mean_edge = w > 0 ? s / w : 1.0;
  return "";
}

long long ref_array_size(const Layout& L, int which) {
  const int d1 = L.dim + 1;
  switch (which) {
    case REF_ELE_PERMUTE: return L.full;
    case REF_ELE_OFFSETS: return L.nparts + 1;
    case REF_VERT_PERMUTE: return L.nv;
    case REF_VERT_IPERMUTE: return L.nv;
    case REF_VERT_OFFSETS: return L.nparts + 1;
    case REF_ELE_AFTER_PERMUTE: return L.full * d1;
    case REF_MEM_LOCATIONS: return L.full * d1;
    case REF_MEM_LOCATION_OFFSETS: return (long long)L.nv + 1;
    case REF_BLOCK_XADJ: return L.nparts + 1;
    case REF_BLOCK_ADJNCY: return (long long)L.padj.size() + (L.has_internal_edge ? 0 : -1);
    case REF_LOCAL_COORDS: return L.full * (L.dim == 3 ? 6 : 3);
  }
  return -1;
}

bool ref_array_copy(const Layout& L, int which, void* dst) {
  const int d1 = L.dim + 1;
  const long long full = L.full;
  int* di = static_cast<int*>(dst);
  switch (which) {
    case REF_ELE_PERMUTE: std::memcpy(dst, L.ele_permute.data(), sizeof(int) * full); return true;
    case REF_ELE_OFFSETS: std::memcpy(dst, L.ele_offsets.data(), sizeof(int) * (L.nparts + 1)); return true;
    case REF_VERT_PERMUTE: std::memcpy(dst, L.vert_permute.data(), sizeof(int) * L.nv); return true;
    case REF_VERT_IPERMUTE: std::memcpy(dst, L.vert_ipermute.data(), sizeof(int) * L.nv); return true;
    case REF_VERT_OFFSETS: std::memcpy(dst, L.vert_offsets.data(), sizeof(int) * (L.nparts + 1)); return true;
    case REF_ELE_AFTER_PERMUTE:
      for (long long c = 0; c < full; ++c)
        for (int k = 0; k < d1; ++k) di[k * full + c] = L.conn[c * d1 + k];
      return true;
    case REF_MEM_LOCATIONS:
    case REF_MEM_LOCATION_OFFSETS: {
      std::vector<int> off((size_t)L.nv + 1, 0);
      for (int k = 0; k < d1; ++k)
        for (long long c = 0; c < full; ++c) off[L.conn[c * d1 + k] + 1]++;
      for (int v = 0; v < L.nv; ++v) off[v + 1] += off[v];
      if (which == REF_MEM_LOCATION_OFFSETS) {
        std::memcpy(dst, off.data(), sizeof(int) * ((size_t)L.nv + 1));
      } else {
        for (int k = 0; k < d1; ++k)
          for (long long c = 0; c < full; ++c) di[off[L.conn[c * d1 + k]]++] = (int)(k * full + c);
      }
      return true;
    }
    case REF_BLOCK_XADJ: {
      // The reference builds block_xadj from the sorted (label, neighbour)
      // pairs with a leading (-1,-1) pair for internal edges; for meshes in
      // which every patch has a neighbour and an internal edge exists this is
      // the plain CSR offset array.
      std::memcpy(dst, L.padj_off.data(), sizeof(int) * (L.nparts + 1));
      return true;
    }
    case REF_BLOCK_ADJNCY: {
      long long n = ref_array_size(L, which);
      if (n < 0) return false;
      std::memcpy(dst, L.padj.data() + (L.has_internal_edge ? 0 : 1), sizeof(int) * n);
      return true;
    }
    case REF_LOCAL_COORDS: {
      float* df = static_cast<float*>(dst);
      for (long long c = 0; c < full; ++c) {
        if (L.dim == 3) {
          float P[4][3], Lc[6];
          for (int k = 0; k < 4; ++k)
            for (int j = 0; j < 3; ++j) P[k][j] = L.xyz_p[(size_t)j * L.nv + L.conn[c * 4 + k]];
          tet_local_coords(P, Lc);
          for (int i = 0; i < 6; ++i) df[i * full + c] = Lc[i];
        } else {
          double P[3][3], Lc[3], sg[2], z[3] = {0, 0, 0};
          for (int k = 0; k < 3; ++k)
            for (int j = 0; j < 3; ++j) P[k][j] = L.xyz_p[(size_t)j * L.nv + L.conn[c * 3 + k]];
          tri_local_coords(P, z, Lc, sg);
          for (int i = 0; i < 3; ++i) df[i * full + c] = (float)Lc[i];
        }
      }
      return true;
    }
  }
  return false;
}

}  // namespace lsgb
