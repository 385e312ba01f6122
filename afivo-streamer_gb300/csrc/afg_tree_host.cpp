// afg_tree_host.cpp -- host-side mesh adjustment for callers without afivo's
// own tree code (the Python host mirror of this repository).  A Fortran
// caller keeps af_adjust_refinement; this file restates it in C++:
//
//   * the flag passes of af_adjust_refinement after consistent_ref_flags
//     (afivo/src/m_af_core.f90:697-1091): the max-level clamp (995-999),
//     ensure_two_one_balance over face neighbours (1015-1055) and
//     handle_derefinement_flags (1057-1088);
//   * the new tree: leaves flagged af_refine get children, the children of
//     parents flagged af_derefine go, then afivo's 2:1 balance over face
//     neighbours; boxes are numbered level by level, level 1 in coordinate
//     order (x fastest), then the children of each refined parent in
//     parent-id order and af_child_dix order; neighbours, neighbor_mat,
//     parent/children and the geometry (r_min, dr) follow, with the
//     operation order of af_init / af_set_coarse_grid / set_child_geometry
//     (m_af_core.f90:166, 255-256, 1210-1213).
//
// Host code only: no CUDA call, usable without a GPU.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <vector>

#include "../../include/afivo_gpu.h"

namespace {

constexpr int kNoBox = 0, kPhys = -1;
constexpr int kRmRef = -1, kKeepRef = 0, kDoRef = 1, kRefine = 2, kDerefine = -2;

struct NewTree {
  int D = 2, n_boxes = 0, highest = 0;
  std::vector<int> lvl, ix, parent, children, neighbors, nbmat;
  std::vector<double> r_min, dr;
  double dr_base[3] = {0, 0, 0};
};

// linear key of 0-based box indices, x fastest
inline int64_t key_of(const int64_t* ix, const int64_t* n, int D) {
  int64_t k = 0;
  for (int d = D - 1; d >= 0; d--) k = k * n[d] + ix[d];
  return k;
}
inline void unkey(int64_t k, const int64_t* n, int D, int64_t* ix) {
  for (int d = 0; d < D; d++) {
    ix[d] = k % n[d];
    k /= n[d];
  }
}
inline long find_sorted(const std::vector<int64_t>& v, int64_t k) {
  auto it = std::lower_bound(v.begin(), v.end(), k);
  return (it != v.end() && *it == k) ? (long)(it - v.begin()) : -1;
}

}  // namespace

struct afg_tree_new {
  NewTree t;
};

extern "C" {

int afg_adjust_refinement(const afg_tree_desc* tr, const int* box_flags, int max_lvl, afg_tree_new** out) {
  if (!tr || !box_flags || !out || max_lvl < 1) return AFG_ERR_ARG;
  *out = nullptr;
  const int D = tr->ndim, nc = tr->n_cell, n = tr->n_boxes, H = tr->highest_lvl;
  if ((D != 2 && D != 3) || nc < 2 || n < 1 || H < 1) return AFG_ERR_ARG;
  const int nch = 1 << D, nnb = 2 * D, nm = D == 2 ? 9 : 27;
  if (!tr->lvl || !tr->parent || !tr->children || !tr->neighbors || !tr->ix || !tr->ids || !tr->ids_off ||
      !tr->leaves || !tr->leaves_off || !tr->parents || !tr->parents_off)
    return AFG_ERR_ARG;
  // level-list offsets: non-negative, non-decreasing, within the box count
  // (every list holds each box at most once)
  for (const int* off : {tr->ids_off, tr->leaves_off, tr->parents_off}) {
    if (off[0] < 0) return AFG_ERR_ARG;
    for (int l = 1; l <= H; l++)
      if (off[l] < off[l - 1] || off[l] > n) return AFG_ERR_ARG;
  }
  // box flags as afivo knows them: remove, keep or refine (af_rm_ref ..
  // af_do_ref); af_adjust_refinement stops on others (m_af_core.f90:993-994)
  for (int b = 0; b < n; b++)
    if (box_flags[b] < kRmRef || box_flags[b] > kDoRef) return AFG_ERR_ARG;
  std::vector<int64_t> f(box_flags, box_flags + n);
  std::vector<char> has_ch(n, 0);
  for (int b = 0; b < n; b++) {
    if (tr->lvl[b] < 1 || tr->lvl[b] > H || tr->parent[b] < 0 || tr->parent[b] > n) return AFG_ERR_ARG;
    for (int d = 0; d < D; d++)
      if (tr->ix[(size_t)b * D + d] < 1) return AFG_ERR_ARG;
    for (int c = 0; c < nch; c++) {
      const int ch = tr->children[(size_t)b * nch + c];
      if (ch < 0 || ch > n) return AFG_ERR_ARG;
      has_ch[b] |= ch > 0;
    }
    for (int q = 0; q < nnb; q++)
      if (tr->neighbors[(size_t)b * nnb + q] < kPhys || tr->neighbors[(size_t)b * nnb + q] > n) return AFG_ERR_ARG;
  }
  auto lvl_list = [&](const int* off, const int* data, int l) {  // l 1-based
    return std::vector<int>(data + off[l - 1], data + off[l]);
  };
  for (int l = 1; l <= H; l++)
    for (const std::vector<int>& v : {lvl_list(tr->ids_off, tr->ids, l), lvl_list(tr->leaves_off, tr->leaves, l),
                                      lvl_list(tr->parents_off, tr->parents, l)})
      for (int id : v)
        if (id < 1 || id > n) return AFG_ERR_ARG;
  // max-level clamp
  if (H >= max_lvl)
    for (int id : lvl_list(tr->ids_off, tr->ids, max_lvl))
      if (f[id - 1] == kDoRef) f[id - 1] = kKeepRef;
  // ensure_two_one_balance (face neighbours)
  for (int l = H; l >= 1; l--)
    for (int id : lvl_list(tr->leaves_off, tr->leaves, l)) {
      const int b = id - 1;
      if (f[b] == kDoRef || f[b] == kRefine) {
        f[b] = kRefine;
        for (int nb = 0; nb < nnb; nb++)
          if (tr->neighbors[(size_t)b * nnb + nb] == kNoBox) {
            const int p = tr->parent[b];
            const int pn = p > 0 ? tr->neighbors[(size_t)(p - 1) * nnb + nb] : 0;
            if (pn <= 0 || pn > n) return AFG_ERR_ARG;   // not 2:1 balanced
            f[pn - 1] = kRefine;
          }
      } else if (f[b] == kRmRef) {
        for (int nb = 0; nb < nnb; nb++) {
          const int nid = tr->neighbors[(size_t)b * nnb + nb];
          if (nid > kNoBox && (has_ch[nid - 1] || f[nid - 1] > kKeepRef)) {
            f[b] = kKeepRef;
            break;
          }
        }
      }
    }
  // handle_derefinement_flags
  for (int l = H - 1; l >= 1; l--)
    for (int id : lvl_list(tr->parents_off, tr->parents, l)) {
      const int* c = tr->children + (size_t)(id - 1) * nch;
      bool all_ch = true, all_rm = true;
      for (int q = 0; q < nch; q++)
        if (c[q] < 1) return AFG_ERR_ARG;   // a parent without all its children
      for (int q = 0; q < nch; q++) {
        all_ch = all_ch && has_ch[c[q] - 1];
        all_rm = all_rm && f[c[q] - 1] == kRmRef;
      }
      if (all_ch) continue;
      if (all_rm && f[id - 1] <= kKeepRef) {
        f[id - 1] = kDerefine;
      } else {
        f[id - 1] = kKeepRef;
        for (int q = 0; q < nch; q++)
          if (f[c[q] - 1] != kDerefine) f[c[q] - 1] = std::max<int64_t>(f[c[q] - 1], kKeepRef);
      }
    }
  // unchanged mesh: no leaf refined and no parent derefined
  bool change = false;
  for (int b = 0; b < n && !change; b++)
    change = (!has_ch[b] && f[b] == kRefine) || (has_ch[b] && f[b] == kDerefine);
  if (!change) return AFG_OK;

  // per level, the keys of the old boxes that keep or get children
  const int L = std::max(max_lvl, H);
  int64_t nx1[3] = {1, 1, 1};
  for (int d = 0; d < D; d++) {
    if (tr->coarse_grid_size[d] % nc) return AFG_ERR_ARG;
    nx1[d] = tr->coarse_grid_size[d] / nc;
  }
  std::vector<std::vector<int64_t>> nlev(L, std::vector<int64_t>(3, 1));
  for (int l = 0; l < L; l++)
    for (int d = 0; d < D; d++) nlev[l][d] = nx1[d] << l;
  std::vector<std::vector<int64_t>> wants(L);
  for (int b = 0; b < n; b++) {
    const bool w = has_ch[b] ? f[b] != kDerefine : f[b] == kRefine;
    if (!w) continue;
    const int l = tr->lvl[b] - 1;
    int64_t ix[3] = {0, 0, 0};
    for (int d = 0; d < D; d++) ix[d] = tr->ix[(size_t)b * D + d] - 1;
    wants[l].push_back(key_of(ix, nlev[l].data(), D));
  }
  for (auto& w : wants) std::sort(w.begin(), w.end());

  // boxes that exist and boxes that are refined, level by level
  std::vector<std::vector<int64_t>> exists(1), refined(L);
  {
    const int64_t n1 = nx1[0] * nx1[1] * nx1[2];
    for (int64_t k = 0; k < n1; k++) exists[0].push_back(k);
  }
  for (int l = 0; l + 1 < L; l++) {
    if (exists[l].empty()) break;
    std::vector<int64_t> nxt;
    for (int64_t k : exists[l]) {
      if (find_sorted(wants[l], k) < 0) continue;
      refined[l].push_back(k);
      int64_t ix[3] = {0, 0, 0}, cix[3] = {0, 0, 0};
      unkey(k, nlev[l].data(), D, ix);
      for (int c = 0; c < nch; c++) {
        for (int d = 0; d < D; d++) cix[d] = 2 * ix[d] + ((c >> d) & 1);
        nxt.push_back(key_of(cix, nlev[l + 1].data(), D));
      }
    }
    std::sort(nxt.begin(), nxt.end());
    exists.push_back(nxt);
  }
  // 2:1 balance over face neighbours, fine to coarse
  for (int l = L - 2; l >= 1; l--) {
    if (refined[l].empty()) continue;
    std::vector<int64_t> add;
    for (int64_t k : refined[l]) {
      int64_t ix[3] = {0, 0, 0};
      unkey(k, nlev[l].data(), D, ix);
      for (int o = -1; o < 2 * D; o++) {   // o = -1: the box itself
        int64_t q[3] = {ix[0], ix[1], ix[2]};
        if (o >= 0) q[o / 2] += (o % 2) ? 1 : -1;
        bool inside = true;
        for (int d = 0; d < D; d++) inside = inside && q[d] >= 0 && q[d] < nlev[l][d];
        if (!inside) continue;
        for (int d = 0; d < D; d++) q[d] /= 2;
        add.push_back(key_of(q, nlev[l - 1].data(), D));
      }
    }
    add.insert(add.end(), refined[l - 1].begin(), refined[l - 1].end());
    std::sort(add.begin(), add.end());
    add.erase(std::unique(add.begin(), add.end()), add.end());
    refined[l - 1] = add;
  }
  exists.resize(1);
  for (int l = 0; l + 1 < L; l++) {
    if (refined[l].empty()) break;
    std::vector<int64_t> nxt;
    for (int64_t k : refined[l]) {
      int64_t ix[3] = {0, 0, 0}, cix[3] = {0, 0, 0};
      unkey(k, nlev[l].data(), D, ix);
      for (int c = 0; c < nch; c++) {
        for (int d = 0; d < D; d++) cix[d] = 2 * ix[d] + ((c >> d) & 1);
        nxt.push_back(key_of(cix, nlev[l + 1].data(), D));
      }
    }
    std::sort(nxt.begin(), nxt.end());
    exists.push_back(nxt);
  }
  const int highest = (int)exists.size();

  // ids: level 1 in key order, then children of refined parents in parent-id order
  std::vector<std::vector<int64_t>> key_by_id(highest);   // keys in id order
  std::vector<int> first_id(highest + 1, 1);
  key_by_id[0] = exists[0];
  int next_id = (int)exists[0].size() + 1;
  first_id[1] = next_id;
  for (int l = 1; l < highest; l++) {
    for (int64_t pk : key_by_id[l - 1]) {
      if (!std::binary_search(refined[l - 1].begin(), refined[l - 1].end(), pk)) continue;
      int64_t ix[3] = {0, 0, 0}, cix[3] = {0, 0, 0};
      unkey(pk, nlev[l - 1].data(), D, ix);
      for (int c = 0; c < nch; c++) {
        for (int d = 0; d < D; d++) cix[d] = 2 * ix[d] + ((c >> d) & 1);
        key_by_id[l].push_back(key_of(cix, nlev[l].data(), D));
      }
    }
    next_id += (int)key_by_id[l].size();
    first_id[l + 1] = next_id;
  }
  NewTree nt;
  nt.D = D;
  nt.n_boxes = next_id - 1;
  nt.highest = highest;
  const int N = nt.n_boxes;
  nt.lvl.assign(N, 0);
  nt.ix.assign((size_t)N * D, 0);
  nt.parent.assign(N, 0);
  nt.children.assign((size_t)N * nch, 0);
  nt.neighbors.assign((size_t)N * nnb, 0);
  nt.nbmat.assign((size_t)N * nm, 0);
  nt.r_min.assign((size_t)N * D, 0.0);
  nt.dr.assign((size_t)N * D, 0.0);

  // geometry of level 1 from the old tree: r_base is r_min of the box at
  // index 1, dr_base its dr; the domain length is recomputed as afivo's
  // af_init does from r_base and r_base + L
  double rb[3] = {0, 0, 0}, drb_old[3] = {0, 0, 0};
  {
    const int* l1 = tr->ids + tr->ids_off[0];
    const int n1 = tr->ids_off[1] - tr->ids_off[0];
    bool found = false;
    for (int q = 0; q < n1 && !found; q++) {
      const int b = l1[q] - 1;
      bool first = true;
      for (int d = 0; d < D; d++) first = first && tr->ix[(size_t)b * D + d] == 1;
      if (first) {
        for (int d = 0; d < D; d++) {
          rb[d] = tr->r_min[(size_t)b * D + d];
          drb_old[d] = tr->dr[(size_t)b * D + d];
        }
        found = true;
      }
    }
    if (!found) return AFG_ERR_ARG;
  }
  for (int d = 0; d < D; d++) {
    const double cgs = (double)tr->coarse_grid_size[d];
    const double dom = drb_old[d] * cgs;
    nt.dr_base[d] = ((rb[d] + dom) - rb[d]) / cgs;
  }
  // neighbour offsets: af_neighb_dix order and neighbor_mat (first index fastest)
  std::vector<std::vector<int>> nb_off, mat_off;
  for (int d = 0; d < D; d++)
    for (int s = -1; s <= 1; s += 2) {
      std::vector<int> v(3, 0);
      v[d] = s;
      nb_off.push_back(v);
    }
  for (int k = 0; k < nm; k++) {
    std::vector<int> v(3, 0);
    int r = k;
    for (int d = 0; d < D; d++) {
      v[d] = r % 3 - 1;
      r /= 3;
    }
    mat_off.push_back(v);
  }
  // per level, the keys sorted with their ids, for lookups
  std::vector<std::vector<std::pair<int64_t, int>>> sorted_ids(highest);
  for (int l = 0; l < highest; l++) {
    const std::vector<int64_t>& kb = key_by_id[l];
    sorted_ids[l].resize(kb.size());
    for (size_t q = 0; q < kb.size(); q++) sorted_ids[l][q] = {kb[q], first_id[l] + (int)q};
    std::sort(sorted_ids[l].begin(), sorted_ids[l].end());
  }
  for (int l = 0; l < highest; l++) {
    const std::vector<int64_t>& kb = key_by_id[l];
    const std::vector<std::pair<int64_t, int>>& sk = sorted_ids[l];
    auto lookup = [&](const int64_t* q) -> int {
      for (int d = 0; d < D; d++)
        if (q[d] < 0 || q[d] >= nlev[l][d]) return kPhys;
      const int64_t k = key_of(q, nlev[l].data(), D);
      auto it = std::lower_bound(sk.begin(), sk.end(), std::make_pair(k, 0));
      return (it != sk.end() && it->first == k) ? it->second : kNoBox;
    };
    for (size_t q = 0; q < kb.size(); q++) {
      const int id = first_id[l] + (int)q, b = id - 1;
      int64_t ix[3] = {0, 0, 0};
      unkey(kb[q], nlev[l].data(), D, ix);
      nt.lvl[b] = l + 1;
      for (int d = 0; d < D; d++) nt.ix[(size_t)b * D + d] = (int)ix[d] + 1;
      for (int o = 0; o < nnb; o++) {
        int64_t p[3] = {ix[0] + nb_off[o][0], ix[1] + nb_off[o][1], ix[2] + nb_off[o][2]};
        nt.neighbors[(size_t)b * nnb + o] = lookup(p);
      }
      for (int o = 0; o < nm; o++) {
        int64_t p[3] = {ix[0] + mat_off[o][0], ix[1] + mat_off[o][1], ix[2] + mat_off[o][2]};
        nt.nbmat[(size_t)b * nm + o] = lookup(p);
      }
      if (l == 0) {
        nt.parent[b] = kNoBox;
        for (int d = 0; d < D; d++) {
          nt.r_min[(size_t)b * D + d] = rb[d] + ((double)ix[d] * nt.dr_base[d]) * nc;
          nt.dr[(size_t)b * D + d] = nt.dr_base[d];
        }
      } else {
        // the parent: the refined box of level l-1 at ix / 2
        int64_t pix[3] = {ix[0] / 2, ix[1] / 2, ix[2] / 2};
        const int64_t pk = key_of(pix, nlev[l - 1].data(), D);
        const std::vector<std::pair<int64_t, int>>& psk = sorted_ids[l - 1];
        auto it = std::lower_bound(psk.begin(), psk.end(), std::make_pair(pk, 0));
        if (it == psk.end() || it->first != pk) return AFG_ERR_STATE;
        const int pid = it->second;
        nt.parent[b] = pid;
        int cnum = 0;
        for (int d = 0; d < D; d++) cnum += (int)((ix[d] & 1) << d);
        nt.children[(size_t)(pid - 1) * nch + cnum] = id;
        for (int d = 0; d < D; d++) {
          const double pdr = nt.dr[(size_t)(pid - 1) * D + d];
          const double dixf = (double)(ix[d] & 1);
          nt.r_min[(size_t)b * D + d] = nt.r_min[(size_t)(pid - 1) * D + d] + ((0.5 * pdr) * dixf) * nc;
          nt.dr[(size_t)b * D + d] = 0.5 * pdr;
        }
      }
    }
  }
  *out = new afg_tree_new{nt};
  return AFG_OK;
}

int afg_tree_new_sizes(const afg_tree_new* t, int* n_boxes, int* highest_lvl) {
  if (!t || !n_boxes || !highest_lvl) return AFG_ERR_ARG;
  *n_boxes = t->t.n_boxes;
  *highest_lvl = t->t.highest;
  return AFG_OK;
}

int afg_tree_new_get(const afg_tree_new* t, int* lvl, int* ix, int* parent, int* children, int* neighbors,
                     int* neighbor_mat, double* r_min, double* dr, double* dr_base) {
  if (!t) return AFG_ERR_ARG;
  const NewTree& n = t->t;
  auto cp = [](const auto& v, auto* dst) {
    if (dst) std::memcpy(dst, v.data(), sizeof(v[0]) * v.size());
  };
  cp(n.lvl, lvl);
  cp(n.ix, ix);
  cp(n.parent, parent);
  cp(n.children, children);
  cp(n.neighbors, neighbors);
  cp(n.nbmat, neighbor_mat);
  cp(n.r_min, r_min);
  cp(n.dr, dr);
  if (dr_base)
    for (int d = 0; d < n.D; d++) dr_base[d] = n.dr_base[d];
  return AFG_OK;
}

void afg_tree_new_free(afg_tree_new* t) { delete t; }

}  // extern "C"
