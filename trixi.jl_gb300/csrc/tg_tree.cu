// Refinement tree of a TreeMesh on the host: construction with refinement
// patches, AMR adaptation and the mesh containers of its leaves.
//
//   tree_mesh.jl:186-215            initialize! (uniform refinement, patches)
//   abstract_tree.jl:35-47          has_neighbor / has_coarse_neighbor
//   abstract_tree.jl:122-130        child order (_child_signs: x fastest)
//   abstract_tree.jl:317-489        refine_unbalanced!, refine!, rebalance!,
//                                   refine_box!, refine_sphere!
//   abstract_tree.jl:516-618        coarsen!
//   abstract_tree.jl:668-674        child_coordinates
//   containers_2d.jl:193-284, 660-810, containers_3d.jl:87-790
//                                   interfaces and L2 mortars of the leaves
//   callbacks_step/amr.jl:244-392   the refine-then-coarsen pass of AMR
//
// Cells are keyed by (level, integer position).  A same-level neighbour
// exists iff its key is present (with periodic wrap per dimension): that is
// what Trixi's neighbour links record.  Trixi stores cells depth-first with
// children right behind their parent, so its elements (the leaves in storage
// order) are the leaves of a depth-first walk with children in child order.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "../../include/trixi_gb300.h"
#include "tg_internal.h"

namespace {

constexpr int kMaxLevel = 15;

// Cell key -> cell id, open addressing with linear probing (capacity a power
// of two, at most half full).  A key is re-pointed when a coarsened cell is
// refined again; keys are never removed (dead cells are told apart by the
// tree's alive flags and dropped when the tree is compacted).
struct CellIndex {
  static constexpr uint64_t kEmpty = ~0ull;  // no key: the level field is at most 15
  std::vector<uint64_t> keys;
  std::vector<int64_t> vals;
  size_t count = 0;

  static size_t hash(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    return (size_t)k;
  }
  void clear(size_t expected) {
    size_t cap = 64;
    while (cap < 2 * expected + 2) cap <<= 1;
    keys.assign(cap, kEmpty);
    vals.assign(cap, -1);
    count = 0;
  }
  void put(uint64_t k, int64_t v) {
    if (2 * (count + 1) > keys.size()) {
      std::vector<uint64_t> ok;
      std::vector<int64_t> ov;
      ok.swap(keys);
      ov.swap(vals);
      clear(ok.size());
      for (size_t i = 0; i < ok.size(); ++i)
        if (ok[i] != kEmpty) put(ok[i], ov[i]);
    }
    const size_t mask = keys.size() - 1;
    for (size_t i = hash(k) & mask;; i = (i + 1) & mask) {
      if (keys[i] == k) {
        vals[i] = v;
        return;
      }
      if (keys[i] == kEmpty) {
        keys[i] = k;
        vals[i] = v;
        ++count;
        return;
      }
    }
  }
  int64_t get(uint64_t k) const {
    if (keys.empty()) return -1;
    const size_t mask = keys.size() - 1;
    for (size_t i = hash(k) & mask;; i = (i + 1) & mask) {
      if (keys[i] == k) return vals[i];
      if (keys[i] == kEmpty) return -1;
    }
  }
};

}  // namespace

struct tg_tree {
  int D = 2;
  bool periodic[3] = {true, true, true};
  double length0 = 0;
  // cells (struct of arrays)
  std::vector<int8_t> level;
  std::vector<int32_t> ix;      // [cell][3]
  std::vector<double> center;   // [cell][3]
  std::vector<int64_t> child0;  // first child, -1 for a leaf
  std::vector<uint8_t> alive;   // 0: a child removed by coarsen!
  int64_t nalive = 0;
  CellIndex index;
  std::vector<int64_t> leaves;  // the elements, in order
  // transfer map of the last adaptation
  std::vector<int64_t> map_source;
  std::vector<int8_t> map_kind;
  // containers of the current leaves (built on demand)
  bool containers_valid = false;
  std::vector<int64_t> if_ids, if_orient, mo_ids, mo_large, mo_orient;

  static uint64_t key(int lev, const int32_t* p) {
    return ((uint64_t)lev << 60) | (uint64_t)p[0] | ((uint64_t)p[1] << 20) | ((uint64_t)p[2] << 40);
  }
  int64_t ncells() const { return (int64_t)level.size(); }
  bool is_leaf(int64_t c) const { return child0[c] < 0; }
  double length(int lev) const { return length0 / (double)(1LL << lev); }

  int64_t find(int lev, const int32_t* p) const {
    const int64_t id = index.get(key(lev, p));
    return id >= 0 && alive[id] ? id : -1;
  }
  int64_t add(int lev, const int32_t* p, const double* c) {
    const int64_t id = ncells();
    level.push_back((int8_t)lev);
    for (int d = 0; d < 3; ++d) {
      ix.push_back(p[d]);
      center.push_back(c[d]);
    }
    child0.push_back(-1);
    alive.push_back(1);
    ++nalive;
    index.put(key(lev, p), id);
    return id;
  }
  // Drops the dead cells: the live ones renumbered breadth-first (children
  // stay consecutive behind their first child), the index rebuilt.  The
  // elements keep their order.
  void compact() {
    const int nch = 1 << D;
    std::vector<int64_t> order{0}, newid(ncells(), -1);
    order.reserve((size_t)nalive);
    newid[0] = 0;
    for (size_t i = 0; i < order.size(); ++i) {
      const int64_t c = order[i];
      if (child0[c] < 0) continue;
      for (int ch = 0; ch < nch; ++ch) {
        newid[child0[c] + ch] = (int64_t)order.size();
        order.push_back(child0[c] + ch);
      }
    }
    const size_t n = order.size();
    std::vector<int8_t> lv(n);
    std::vector<int32_t> p(3 * n);
    std::vector<double> x(3 * n);
    std::vector<int64_t> c0(n);
    for (size_t i = 0; i < n; ++i) {
      const int64_t c = order[i];
      lv[i] = level[c];
      for (int d = 0; d < 3; ++d) {
        p[3 * i + d] = ix[3 * c + d];
        x[3 * i + d] = center[3 * c + d];
      }
      c0[i] = child0[c] < 0 ? -1 : newid[child0[c]];
    }
    level.swap(lv);
    ix.swap(p);
    center.swap(x);
    child0.swap(c0);
    alive.assign(n, 1);
    nalive = (int64_t)n;
    index.clear(n);
    for (size_t i = 0; i < n; ++i) index.put(key(level[i], &ix[3 * i]), (int64_t)i);
    for (int64_t& c : leaves) c = newid[c];
    containers_valid = false;
  }
  // same-level neighbour across face `dir` (0: -x, 1: +x, 2: -y, ...), or -1
  int64_t neighbour(int64_t c, int dir) const {
    int32_t p[3] = {ix[3 * c], ix[3 * c + 1], ix[3 * c + 2]};
    const int d = dir >> 1, lev = level[c];
    const int32_t M = 1 << lev;
    p[d] += (dir & 1) ? 1 : -1;
    if (p[d] < 0 || p[d] >= M) {
      if (!periodic[d]) return -1;
      p[d] = (p[d] + M) % M;
    }
    return find(lev, p);
  }
  int64_t parent(int64_t c) const {
    if (level[c] == 0) return -1;
    const int32_t p[3] = {ix[3 * c] >> 1, ix[3 * c + 1] >> 1, ix[3 * c + 2] >> 1};
    return find(level[c] - 1, p);
  }
  // init_child! with child_coordinates: centre + sign * (parent length / 2) / 2
  void refine_cell(int64_t c) {
    const int lev = level[c];
    const double half_child = length(lev) / 4;
    const int32_t p0[3] = {ix[3 * c], ix[3 * c + 1], ix[3 * c + 2]};
    const double c0[3] = {center[3 * c], center[3 * c + 1], center[3 * c + 2]};
    const int64_t first = ncells();
    for (int ch = 0; ch < (1 << D); ++ch) {
      int32_t p[3] = {0, 0, 0};
      double x[3] = {0, 0, 0};
      for (int d = 0; d < D; ++d) {
        const int bit = (ch >> d) & 1;
        p[d] = 2 * p0[d] + bit;
        x[d] = c0[d] + (bit ? 1.0 : -1.0) * half_child;
      }
      add(lev + 1, p, x);
    }
    child0[c] = first;
  }
  // All or nothing: no cell is refined when one is at the maximum level
  // (rebalance! only marks cells coarser than the ones that triggered it, so a
  // refine! that passes this check for its own cells cannot fail later).
  bool refine_unbalanced(std::vector<int64_t>& ids) {
    std::sort(ids.begin(), ids.end());
    ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
    for (int64_t c : ids)
      if (level[c] >= kMaxLevel) return false;
    for (int64_t c : ids) refine_cell(c);
    return true;
  }
  // refine!(t, cell_ids): the leaves given, then rebalance! until no two face
  // neighbours differ by more than one level
  bool refine(std::vector<int64_t> ids) {
    if (!refine_unbalanced(ids)) return false;
    std::vector<int64_t> marks;
    while (!ids.empty()) {
      marks.clear();
      for (int64_t c : ids)
        for (int dir = 0; dir < 2 * D; ++dir) {
          if (neighbour(c, dir) >= 0) continue;
          const int64_t p = parent(c);
          if (p < 0) continue;
          const int64_t pn = neighbour(p, dir);
          if (pn >= 0) marks.push_back(pn);
        }
      ids.swap(marks);
      if (!refine_unbalanced(ids)) return false;
    }
    return true;
  }
  // coarsen!(t, cell_ids): parents from the highest level down; a parent is
  // kept when one of its children has a same-level neighbour with children
  // across a face not shared with a sibling (the 2:1 rule).  Returns the
  // coarsened parents with their former first child.
  std::vector<std::pair<int64_t, int64_t>> coarsen(std::vector<int64_t> ids) {
    std::stable_sort(ids.begin(), ids.end(),
                     [&](int64_t a, int64_t b) { return level[a] < level[b]; });
    std::vector<std::pair<int64_t, int64_t>> done;
    while (!ids.empty()) {
      const int64_t c = ids.back();
      ids.pop_back();
      const int64_t first = child0[c];
      bool skip = false;
      for (int ch = 0; ch < (1 << D) && !skip; ++ch)
        for (int dir = 0; dir < 2 * D; ++dir) {
          if (((ch >> (dir >> 1)) & 1) != (dir & 1)) continue;  // a sibling's face
          const int64_t nb = neighbour(first + ch, dir);
          if (nb >= 0 && !is_leaf(nb)) {
            skip = true;
            break;
          }
        }
      if (skip) continue;
      for (int ch = 0; ch < (1 << D); ++ch) alive[first + ch] = 0;
      nalive -= 1 << D;
      child0[c] = -1;
      done.emplace_back(c, first);
    }
    return done;
  }
  void rebuild_leaves() {
    leaves.clear();
    std::vector<int64_t> stack{0};
    const int nch = 1 << D;
    while (!stack.empty()) {
      const int64_t c = stack.back();
      stack.pop_back();
      if (child0[c] < 0) {
        leaves.push_back(c);
      } else {
        for (int ch = nch - 1; ch >= 0; --ch) stack.push_back(child0[c] + ch);
      }
    }
    containers_valid = false;
  }
  // init_interfaces! and init_mortars! of the leaves
  void build_containers() {
    if (containers_valid) return;
    std::vector<int64_t> elem(ncells(), -1);
    for (int64_t e = 0; e < (int64_t)leaves.size(); ++e) elem[leaves[e]] = e;
    if_ids.clear();
    if_orient.clear();
    mo_ids.clear();
    mo_large.clear();
    mo_orient.clear();
    for (int64_t e = 0; e < (int64_t)leaves.size(); ++e)
      for (int d = 0; d < D; ++d) {
        const int64_t n = neighbour(leaves[e], 2 * d + 1);
        if (n < 0 || !is_leaf(n)) continue;
        if_ids.push_back(e + 1);
        if_ids.push_back(elem[n] + 1);
        if_orient.push_back(d + 1);
      }
    for (int64_t e = 0; e < (int64_t)leaves.size(); ++e)
      for (int dir = 0; dir < 2 * D; ++dir) {
        const int64_t n = neighbour(leaves[e], dir);
        if (n < 0 || is_leaf(n)) continue;
        const int d = dir >> 1, want = (dir & 1) ? 0 : 1;
        for (int ch = 0; ch < (1 << D); ++ch)
          if (((ch >> d) & 1) == want) mo_ids.push_back(elem[child0[n] + ch] + 1);
        mo_ids.push_back(e + 1);
        mo_large.push_back((dir & 1) ? 1 : 2);
        mo_orient.push_back(d + 1);
      }
    containers_valid = true;
  }
};

namespace {

int tree_fail(const char* msg) {
  tg::set_thread_error(msg);
  return TG_ERR_INVALID_ARGUMENT;
}

}  // namespace

extern "C" {

int tg_tree_create(int32_t ndims, int32_t initial_refinement_level, const double* coordinates_min,
                   const double* coordinates_max, const int32_t* periodicity, tg_tree** out) {
  if (!out || !coordinates_min || !coordinates_max) return tree_fail("tree: null argument");
  *out = nullptr;
  if (ndims != 2 && ndims != 3) return tree_fail("tree: ndims must be 2 or 3");
  if (initial_refinement_level < 0 || initial_refinement_level > (ndims == 2 ? 13 : 9))
    return tree_fail("tree: initial_refinement_level out of range");
  const double len = coordinates_max[0] - coordinates_min[0];
  if (!(len > 0)) return tree_fail("tree: coordinates_min must be below coordinates_max");
  tg_tree* t = new tg_tree();
  t->D = ndims;
  t->length0 = len;
  double c0[3] = {0, 0, 0};
  for (int d = 0; d < ndims; ++d) {
    c0[d] = (coordinates_min[d] + coordinates_max[d]) / 2;
    t->periodic[d] = periodicity ? periodicity[d] != 0 : true;
  }
  const int64_t expect = (int64_t)1 << (ndims * initial_refinement_level);
  t->index.clear((size_t)(expect * 1.5) + 16);
  const int32_t root[3] = {0, 0, 0};
  t->add(0, root, c0);
  t->rebuild_leaves();
  for (int l = 0; l < initial_refinement_level; ++l) {
    std::vector<int64_t> all = t->leaves;
    t->refine(all);
    t->rebuild_leaves();
  }
  *out = t;
  return TG_OK;
}

int tg_tree_destroy(tg_tree* t) {
  delete t;
  return TG_OK;
}

int tg_tree_refine_patch(tg_tree* t, int32_t type, const double* a, const double* b,
                         double radius) {
  if (!t || !a || (type == 0 && !b) || (type != 0 && type != 1))
    return tree_fail("tree: invalid refinement patch");
  std::vector<int64_t> sel;
  for (int64_t c : t->leaves) {
    const double* x = &t->center[3 * c];
    bool in = true;
    if (type == 0) {
      for (int d = 0; d < t->D; ++d) in = in && a[d] < x[d] && b[d] > x[d];
    } else {
      double r2 = 0;
      for (int d = 0; d < t->D; ++d) r2 += (x[d] - a[d]) * (x[d] - a[d]);
      in = r2 < radius * radius;
    }
    if (in) sel.push_back(c);
  }
  if (sel.empty()) return TG_OK;
  if (!t->refine(sel)) return tree_fail("tree: refinement beyond the maximum level");
  t->rebuild_leaves();
  return TG_OK;
}

int tg_tree_nelements(const tg_tree* t, int64_t* n) {
  if (!t || !n) return TG_ERR_INVALID_ARGUMENT;
  *n = (int64_t)t->leaves.size();
  return TG_OK;
}

int tg_tree_elements(const tg_tree* t, int32_t* levels, double* centers) {
  if (!t) return TG_ERR_INVALID_ARGUMENT;
  for (size_t e = 0; e < t->leaves.size(); ++e) {
    const int64_t c = t->leaves[e];
    if (levels) levels[e] = t->level[c];
    if (centers)
      for (int d = 0; d < t->D; ++d) centers[e * t->D + d] = t->center[3 * c + d];
  }
  return TG_OK;
}

int tg_tree_counts(tg_tree* t, int64_t* ninterfaces, int64_t* nmortars) {
  if (!t) return TG_ERR_INVALID_ARGUMENT;
  t->build_containers();
  if (ninterfaces) *ninterfaces = (int64_t)t->if_orient.size();
  if (nmortars) *nmortars = (int64_t)t->mo_orient.size();
  return TG_OK;
}

int tg_tree_interfaces(tg_tree* t, int64_t* neighbor_ids, int64_t* orientations) {
  if (!t || !neighbor_ids || !orientations) return TG_ERR_INVALID_ARGUMENT;
  t->build_containers();
  std::memcpy(neighbor_ids, t->if_ids.data(), sizeof(int64_t) * t->if_ids.size());
  std::memcpy(orientations, t->if_orient.data(), sizeof(int64_t) * t->if_orient.size());
  return TG_OK;
}

int tg_tree_mortars(tg_tree* t, int64_t* neighbor_ids, int64_t* large_sides,
                    int64_t* orientations) {
  if (!t || !neighbor_ids || !large_sides || !orientations) return TG_ERR_INVALID_ARGUMENT;
  t->build_containers();
  std::memcpy(neighbor_ids, t->mo_ids.data(), sizeof(int64_t) * t->mo_ids.size());
  std::memcpy(large_sides, t->mo_large.data(), sizeof(int64_t) * t->mo_large.size());
  std::memcpy(orientations, t->mo_orient.data(), sizeof(int64_t) * t->mo_orient.size());
  return TG_OK;
}

int tg_tree_adapt(tg_tree* t, const int8_t* controller_value, int32_t only_refine,
                  int32_t only_coarsen, int32_t* changed) {
  if (!t || !controller_value || !changed) return TG_ERR_INVALID_ARGUMENT;
  *changed = 0;
  const int nch = 1 << t->D;
  const std::vector<int64_t> old = t->leaves;
  std::vector<int64_t> to_refine, to_coarsen;
  for (size_t e = 0; e < old.size(); ++e) {
    if (controller_value[e] > 0) to_refine.push_back(old[e]);
    if (controller_value[e] < 0) to_coarsen.push_back(old[e]);
  }
  bool any = false;
  if (!only_coarsen && !to_refine.empty()) {
    if (!t->refine(to_refine)) return tree_fail("tree: refinement beyond the maximum level");
    any = true;
  }
  std::vector<std::pair<int64_t, int64_t>> coarsened;
  if (!only_refine && !to_coarsen.empty()) {
    std::unordered_map<int64_t, int> count;
    std::vector<int64_t> parents;
    for (int64_t c : to_coarsen) {
      if (t->level[c] == 0 || !t->is_leaf(c)) continue;
      const int64_t p = t->parent(c);
      if (++count[p] == nch) parents.push_back(p);
    }
    std::sort(parents.begin(), parents.end());
    coarsened = t->coarsen(parents);
    any = any || !coarsened.empty();
  }
  if (!any) return TG_OK;
  // transfer map: old element of each cell that was a leaf
  std::vector<int64_t> elem(t->ncells(), -1);
  for (int64_t e = 0; e < (int64_t)old.size(); ++e) elem[old[e]] = e;
  std::vector<int64_t> first_child(t->ncells(), -1);
  for (const auto& pc : coarsened) first_child[pc.first] = pc.second;
  t->rebuild_leaves();
  const size_t E = t->leaves.size();
  t->map_source.assign(E, 0);
  t->map_kind.assign(E, 0);
  for (size_t e = 0; e < E; ++e) {
    const int64_t c = t->leaves[e];
    if (elem[c] >= 0) {
      t->map_source[e] = elem[c];
    } else if (first_child[c] >= 0) {
      t->map_source[e] = elem[first_child[c]];
      t->map_kind[e] = -1;
    } else {
      const int64_t p = t->parent(c);
      t->map_source[e] = elem[p];
      t->map_kind[e] = (int8_t)(1 + (c - t->child0[p]));
    }
  }
  // the cells coarsened away stay in the arrays until they outnumber the live
  // ones
  if (t->ncells() > 2 * t->nalive) t->compact();
  *changed = 1;
  return TG_OK;
}

int tg_tree_transfer_map(const tg_tree* t, int64_t* source_element, int8_t* kind) {
  if (!t || !source_element || !kind) return TG_ERR_INVALID_ARGUMENT;
  if (t->map_source.size() != t->leaves.size())
    return tree_fail("tree: no transfer map for the current elements");
  std::memcpy(source_element, t->map_source.data(), sizeof(int64_t) * t->map_source.size());
  std::memcpy(kind, t->map_kind.data(), t->map_kind.size());
  return TG_OK;
}

}  // extern "C"
