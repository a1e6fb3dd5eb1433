// ORACLE — test infrastructure only (see oracle_core.hpp).
//
// The reference's sparse volume: a VDB-like static tree
// RootNode -> InternalNode<5> -> InternalNode<4> -> LeafNode<3>
// (voxel/volume/mod.rs:8), restated with the same slot, tile and mask
// semantics, including the flood-fill and CSG quirks that change results:
//  * an internal node's last_value_sign() reads its last child's FIRST value
//    (internal_node/flood_fill.rs:103-109);
//  * flood fill writes a signed "far" value into inactive tile slots without
//    setting value_mask (internal_node/flood_fill.rs:64-69);
//  * leaf CSG ORs the value masks for all three operations (leaf_node/csg.rs).
#pragma once

#include "oracle_core.hpp"

namespace orc {

// ----------------------------------------------------------------- leaf --
// leaf_node/{mod.rs, tree_node.rs, flood_fill.rs, csg.rs}
template <int LOG2>
struct Leaf {
  static constexpr int BR = LOG2;
  static constexpr int TOTAL = LOG2;
  static constexpr int N = 1 << (3 * LOG2);
  static constexpr int RES = 1 << LOG2;
  static constexpr bool IS_LEAF = true;
  using LeafT = Leaf;

  I3 origin{0, 0, 0};
  float values[N];
  Bits<N> mask;

  explicit Leaf(I3 o) : origin(o) {
    for (int i = 0; i < N; ++i) values[i] = 0.0f;
  }
  static int offset(const I3& i) {
    const int64_t m = (int64_t(1) << TOTAL) - 1;
    return int(((i.x & m) << (BR + BR)) + ((i.y & m) << BR) + (i.z & m));
  }
  static std::unique_ptr<Leaf> empty(I3 o) { return std::make_unique<Leaf>(o); }

  const float* at(const I3& i) const {
    int o = offset(i);
    return mask.at(o) ? &values[o] : nullptr;
  }
  float* at_mut(const I3& i) {
    int o = offset(i);
    return mask.at(o) ? &values[o] : nullptr;
  }
  void insert(const I3& i, float v) {
    int o = offset(i);
    mask.on(o);
    values[o] = v;
  }
  void remove(const I3& i) { mask.off(offset(i)); }
  bool is_empty() const { return mask.is_empty(); }
  void fill(float v) {
    mask.on_all();
    for (int i = 0; i < N; ++i) values[i] = v;
  }
  void clear() { mask.off_all(); }
  std::unique_ptr<Leaf> clone() const {
    auto c = std::make_unique<Leaf>(origin);
    c->mask = mask;
    std::memcpy(c->values, values, sizeof values);
    return c;
  }
  template <class F>
  void remove_if(F pred) {
    for (int i = 0; i < N; ++i)
      if (mask.at(i) && pred(values[i])) mask.off(i);
  }
  void remove_empty_branches() {}
  template <class F>
  void visit_values_mut(F f) {
    for (int i = 0; i < N; ++i)
      if (mask.at(i)) f(values[i]);
  }
  template <class FD, class FT>
  void visit_leafs(FD dense, FT /*tile*/) const { dense(*this); }
  const Leaf* leaf_at(const I3&) const { return this; }

  // flood_fill.rs:12-50
  void flood_fill() {
    if (mask.is_full()) return;
    int first = mask.find_first_on();
    if (first < 0) return;
    Sign i = sign_of(values[first]);
    for (int x = 0; x < RES; ++x) {
      int x00 = x << (BR + BR);
      if (mask.at(x00)) i = sign_of(values[x00]);
      Sign j = i;
      for (int y = 0; y < RES; ++y) {
        int xy0 = x00 + (y << BR);
        if (mask.at(xy0)) j = sign_of(values[xy0]);
        Sign k = j;
        for (int z = 0; z < RES; ++z) {
          int xyz = xy0 + z;
          if (mask.at(xyz)) {
            k = sign_of(values[xyz]);
          } else {
            values[xyz] = FAR;
            set_sign(values[xyz], k);
          }
        }
      }
    }
  }
  void fill_with_sign(Sign s) {
    for (int i = 0; i < N; ++i) {
      if (!mask.at(i)) values[i] = FAR;
      set_sign(values[i], s);
    }
  }
  Sign first_value_sign() const { return sign_of(values[0]); }
  Sign last_value_sign() const { return sign_of(values[N - 1]); }
  Sign sign_at(const I3& i) const { return sign_of(values[offset(i)]); }

  // utils.rs:38-62 partial_min / partial_max (ties and NaN pick b)
  static float pmin(float a, float b) { return (a < b) ? a : b; }
  static float pmax(float a, float b) { return (a > b) ? a : b; }
  void csg_union(std::unique_ptr<Leaf> o) {
    for (int i = 0; i < N; ++i) values[i] = pmin(values[i], o->values[i]);
    mask |= o->mask;
  }
  void csg_subtract(std::unique_ptr<Leaf> o) {
    for (int i = 0; i < N; ++i) values[i] = pmax(values[i], -o->values[i]);
    mask |= o->mask;
  }
  void csg_intersect(std::unique_ptr<Leaf> o) {
    for (int i = 0; i < N; ++i) values[i] = pmax(values[i], o->values[i]);
    mask |= o->mask;
  }
  void flip_signs() {
    for (int i = 0; i < N; ++i) values[i] = -values[i];
  }
};

// ------------------------------------------------------------- internal --
// internal_node/{mod.rs, tree_node.rs, flood_fill.rs, csg.rs}
template <int LOG2, class C>
struct Internal {
  static constexpr int BR = LOG2;
  static constexpr int TOTAL = LOG2 + C::TOTAL;
  static constexpr int N = 1 << (3 * LOG2);
  static constexpr int DIM = 1 << LOG2;
  static constexpr bool IS_LEAF = false;
  using Child = C;
  using LeafT = typename C::LeafT;

  I3 origin{0, 0, 0};
  Bits<N> child_mask, value_mask;
  std::vector<std::unique_ptr<C>> childs;
  std::vector<float> tiles;  // the tile half of the child union

  explicit Internal(I3 o) : origin(o), childs(N), tiles(N, 0.0f) {}
  static std::unique_ptr<Internal> empty(I3 o) { return std::make_unique<Internal>(o); }

  static int offset(const I3& i) {
    const int64_t m = (int64_t(1) << TOTAL) - 1;
    return int((((i.x & m) >> C::TOTAL) << (BR + BR)) + (((i.y & m) >> C::TOTAL) << BR) +
               ((i.z & m) >> C::TOTAL));
  }
  I3 offset_to_global(int off) const {
    int64_t x = off >> (2 * BR);
    off &= (1 << (2 * BR)) - 1;
    int64_t y = off >> BR;
    int64_t z = off & ((1 << BR) - 1);
    return i3((x << C::TOTAL) + origin.x, (y << C::TOTAL) + origin.y, (z << C::TOTAL) + origin.z);
  }
  bool is_branch(int o) const { return child_mask.at(o); }
  bool is_tile(int o) const { return !child_mask.at(o) && value_mask.at(o); }

  C* add_branch(int o) {
    if (child_mask.at(o)) return childs[o].get();
    child_mask.on(o);
    value_mask.off(o);
    childs[o] = C::empty(offset_to_global(o));
    return childs[o].get();
  }
  std::unique_ptr<C> remove_branch(int o) {
    if (!child_mask.at(o)) return nullptr;
    child_mask.off(o);
    return std::move(childs[o]);
  }
  void remove_child(int o) {
    if (child_mask.at(o)) {
      child_mask.off(o);
      childs[o].reset();
    } else if (value_mask.at(o)) {
      value_mask.off(o);
    }
  }

  const float* at(const I3& i) const {
    int o = offset(i);
    if (child_mask.at(o)) return childs[o]->at(i);
    if (value_mask.at(o)) return &tiles[o];
    return nullptr;
  }
  void insert(const I3& i, float v) {
    int o = offset(i);
    if (child_mask.at(o)) {
      childs[o]->insert(i, v);
    } else if (value_mask.at(o)) {
      float tv = tiles[o];
      if (tv == v) return;
      C* b = add_branch(o);
      b->fill(tv);
      b->insert(i, v);
    } else {
      add_branch(o)->insert(i, v);
    }
  }
  void remove(const I3& i) {
    int o = offset(i);
    if (child_mask.at(o)) {
      childs[o]->remove(i);
      if (childs[o]->is_empty()) remove_branch(o);
    } else if (value_mask.at(o)) {
      float tv = tiles[o];
      C* b = add_branch(o);
      b->fill(tv);
      b->remove(i);
    }
  }
  bool is_empty() const { return child_mask.is_empty() && value_mask.is_empty(); }
  void fill(float v) {
    clear();
    value_mask.on_all();
    for (int o = 0; o < N; ++o) tiles[o] = v;
  }
  void clear() {
    for (int o = 0; o < N; ++o)
      if (child_mask.at(o)) childs[o].reset();
    child_mask.off_all();
    value_mask.off_all();
  }
  std::unique_ptr<Internal> clone() const {
    auto c = std::make_unique<Internal>(origin);
    c->child_mask = child_mask;
    c->value_mask = value_mask;
    c->tiles = tiles;
    for (int o = 0; o < N; ++o)
      if (child_mask.at(o)) c->childs[o] = childs[o]->clone();
    return c;
  }
  // Visits children in slot order (tree_node.rs:229-239).
  template <class FD, class FT>
  void visit_leafs(FD dense, FT tile) const {
    for (int o = 0; o < N; ++o) {
      if (child_mask.at(o))
        childs[o]->visit_leafs(dense, tile);
      else if (value_mask.at(o))
        tile(offset_to_global(o), int(int64_t(1) << C::TOTAL), tiles[o]);
    }
  }
  template <class F>
  void visit_values_mut(F f) {
    for (int o = 0; o < N; ++o) {
      if (child_mask.at(o))
        childs[o]->visit_values_mut(f);
      else if (value_mask.at(o))
        f(tiles[o]);
    }
  }
  const LeafT* leaf_at(const I3& i) const {
    int o = offset(i);
    if (child_mask.at(o)) return childs[o]->leaf_at(i);
    return nullptr;
  }
  std::unique_ptr<LeafT> take_leaf_at(const I3& i) {
    int o = offset(i);
    if (!child_mask.at(o)) return nullptr;
    if constexpr (C::IS_LEAF) {
      return remove_branch(o);
    } else {
      return childs[o]->take_leaf_at(i);
    }
  }
  void insert_leaf_at(std::unique_ptr<LeafT> leaf) {
    I3 idx = leaf->origin;
    int o = offset(idx);
    value_mask.off(o);
    if constexpr (C::IS_LEAF) {
      remove_branch(o);
      child_mask.on(o);
      value_mask.off(o);
      childs[o] = std::move(leaf);
    } else {
      if (child_mask.at(o))
        childs[o]->insert_leaf_at(std::move(leaf));
      else
        add_branch(o)->insert_leaf_at(std::move(leaf));
    }
  }
  void remove_empty_branches() {
    for (int o = 0; o < N; ++o) {
      if (child_mask.at(o)) {
        childs[o]->remove_empty_branches();
        if (childs[o]->is_empty()) remove_branch(o);
      }
    }
  }
  template <class F>
  void remove_if(F pred) {
    for (int o = 0; o < N; ++o) {
      if (child_mask.at(o)) {
        childs[o]->remove_if(pred);
        if (childs[o]->is_empty()) remove_branch(o);
      } else if (value_mask.at(o)) {
        if (pred(tiles[o])) value_mask.off(o);
      }
    }
  }

  // flood_fill.rs:17-83
  Sign child_last_sign(int o) const { return childs[o]->last_value_sign(); }
  void flood_fill() {
    if (value_mask.is_full()) return;
    for (int o = 0; o < N; ++o)
      if (child_mask.at(o)) childs[o]->flood_fill();
    int fv = value_mask.find_first_on();
    int fb = child_mask.find_first_on();
    Sign i;
    if (fv >= 0 && fb >= 0 && fv <= fb)
      i = sign_of(tiles[fv]);
    else if (fv >= 0 && fb >= 0)
      i = childs[fb]->first_value_sign();
    else if (fv >= 0)
      i = sign_of(tiles[fv]);
    else if (fb >= 0)
      i = childs[fb]->first_value_sign();
    else
      return;
    for (int x = 0; x < DIM; ++x) {
      int x00 = x << (BR + BR);
      if (child_mask.at(x00))
        i = child_last_sign(x00);
      else if (value_mask.at(x00))
        i = sign_of(tiles[x00]);
      Sign j = i;
      for (int y = 0; y < DIM; ++y) {
        int xy0 = x00 + (y << BR);
        if (child_mask.at(xy0))
          j = child_last_sign(xy0);
        else if (value_mask.at(xy0))
          j = sign_of(tiles[xy0]);
        Sign k = j;
        for (int z = 0; z < DIM; ++z) {
          int xyz = xy0 + z;
          if (child_mask.at(xyz))
            k = child_last_sign(xyz);
          else if (value_mask.at(xyz))
            k = sign_of(tiles[xyz]);
          else {
            tiles[xyz] = FAR;
            set_sign(tiles[xyz], k);
          }
        }
      }
    }
  }
  void fill_with_sign(Sign s) {
    if (value_mask.is_full()) return;
    for (int o = 0; o < N; ++o) {
      if (child_mask.at(o))
        childs[o]->fill_with_sign(s);
      else if (value_mask.at(o))
        set_sign(tiles[o], s);
      else {
        tiles[o] = FAR;
        set_sign(tiles[o], s);
      }
    }
  }
  Sign first_value_sign() const {
    if (child_mask.at(0)) return childs[0]->first_value_sign();
    return sign_of(tiles[0]);
  }
  // The reference reads the first value of the last child here.
  Sign last_value_sign() const {
    if (child_mask.at(N - 1)) return childs[N - 1]->first_value_sign();
    return sign_of(tiles[N - 1]);
  }
  Sign sign_at(const I3& i) const {
    int o = offset(i);
    if (child_mask.at(o)) return childs[o]->sign_at(i);
    return sign_of(tiles[o]);
  }

  // csg.rs:20-52
  bool is_inside_tile(int o) const { return !child_mask.at(o) && sign_of(tiles[o]) == Sign::Neg; }
  bool is_outside_tile(int o) const { return !child_mask.at(o) && sign_of(tiles[o]) == Sign::Pos; }
  void take_child(Internal& other, int o) {
    if (other.child_mask.at(o)) {
      other.child_mask.set(o, child_mask.at(o));
      other.value_mask.set(o, value_mask.at(o));
      child_mask.on(o);
      value_mask.off(o);
      std::swap(childs[o], other.childs[o]);
      std::swap(tiles[o], other.tiles[o]);
    }
  }
  void make_child_inside(int o) {
    remove_child(o);
    value_mask.on(o);
    tiles[o] = -FAR;
  }
  // csg.rs:68-162
  void csg_union(std::unique_ptr<Internal> other) {
    for (int o = 0; o < N; ++o) {
      if (is_inside_tile(o)) continue;
      if (other->is_inside_tile(o)) { make_child_inside(o); continue; }
      if (is_outside_tile(o)) { take_child(*other, o); continue; }
      if (child_mask.at(o) && other->child_mask.at(o)) {
        auto ob = other->remove_branch(o);
        childs[o]->csg_union(std::move(ob));
        if (childs[o]->is_empty()) make_child_inside(o);
      } else {
        other->remove_child(o);
      }
    }
  }
  void csg_subtract(std::unique_ptr<Internal> other) {
    for (int o = 0; o < N; ++o) {
      if (is_outside_tile(o) || other->is_outside_tile(o)) continue;
      if (other->is_inside_tile(o)) { remove_child(o); continue; }
      if (is_inside_tile(o)) {
        take_child(*other, o);
        if (child_mask.at(o))
          childs[o]->flip_signs();
        else if (value_mask.at(o))
          tiles[o] = -tiles[o];
        continue;
      }
      if (child_mask.at(o) && other->child_mask.at(o)) {
        auto ob = other->remove_branch(o);
        childs[o]->csg_subtract(std::move(ob));
      } else {
        other->remove_child(o);
      }
    }
  }
  void csg_intersect(std::unique_ptr<Internal> other) {
    for (int o = 0; o < N; ++o) {
      if (is_outside_tile(o) || other->is_inside_tile(o)) continue;
      if (other->is_outside_tile(o)) { remove_child(o); continue; }
      if (is_inside_tile(o)) { take_child(*other, o); continue; }
      if (child_mask.at(o) && other->child_mask.at(o)) {
        auto ob = other->remove_branch(o);
        childs[o]->csg_intersect(std::move(ob));
      } else {
        other->remove_child(o);
      }
    }
  }
  void flip_signs() {
    for (int o = 0; o < N; ++o) {
      if (child_mask.at(o))
        childs[o]->flip_signs();
      else if (value_mask.at(o))
        tiles[o] = -tiles[o];
    }
  }
};

// ----------------------------------------------------------------- root --
// root_node/{mod.rs, tree_node.rs, flood_fill.rs, csg.rs}; keys are ordered
// lexicographically (x, y, z) like RootKey's Ord.
template <class C>
struct Root {
  static constexpr bool IS_LEAF = false;
  using Child = C;
  using LeafT = typename C::LeafT;
  static constexpr int64_t CRES = int64_t(1) << C::TOTAL;
  std::map<I3, std::unique_ptr<C>> root;

  static I3 root_key(const I3& i) {
    const int64_t m = ~(CRES - 1);
    return i3(i.x & m, i.y & m, i.z & m);
  }
  const float* at(const I3& i) const {
    auto it = root.find(root_key(i));
    return it == root.end() ? nullptr : it->second->at(i);
  }
  void insert(const I3& i, float v) {
    I3 k = root_key(i);
    auto& slot = root[k];
    if (!slot) slot = C::empty(k);
    slot->insert(i, v);
  }
  void remove(const I3& i) {
    I3 k = root_key(i);
    auto it = root.find(k);
    if (it == root.end()) return;
    it->second->remove(i);
    if (it->second->is_empty()) root.erase(it);
  }
  bool is_empty() const {
    for (auto& kv : root)
      if (!kv.second->is_empty()) return false;
    return true;
  }
  void clear() { root.clear(); }
  std::unique_ptr<Root> clone() const {
    auto c = std::make_unique<Root>();
    for (auto& kv : root) c->root[kv.first] = kv.second->clone();
    return c;
  }
  template <class FD, class FT>
  void visit_leafs(FD dense, FT tile) const {
    for (auto& kv : root) kv.second->visit_leafs(dense, tile);
  }
  template <class F>
  void visit_values_mut(F f) {
    for (auto& kv : root) kv.second->visit_values_mut(f);
  }
  const LeafT* leaf_at(const I3& i) const {
    auto it = root.find(root_key(i));
    return it == root.end() ? nullptr : it->second->leaf_at(i);
  }
  std::unique_ptr<LeafT> take_leaf_at(const I3& i) {
    auto it = root.find(root_key(i));
    if (it == root.end()) return nullptr;
    if constexpr (C::IS_LEAF) {
      return nullptr;  // not reached with Internal children
    } else {
      return it->second->take_leaf_at(i);
    }
  }
  void insert_leaf_at(std::unique_ptr<LeafT> leaf) {
    I3 k = root_key(leaf->origin);
    auto& slot = root[k];
    if (!slot) slot = C::empty(k);
    slot->insert_leaf_at(std::move(leaf));
  }
  void remove_empty_branches() {
    for (auto it = root.begin(); it != root.end();) {
      it->second->remove_empty_branches();
      if (it->second->is_empty())
        it = root.erase(it);
      else
        ++it;
    }
  }
  template <class F>
  void remove_if(F pred) {
    for (auto it = root.begin(); it != root.end();) {
      it->second->remove_if(pred);
      if (it->second->is_empty())
        it = root.erase(it);
      else
        ++it;
    }
  }
  // flood_fill.rs:8-42
  void flood_fill() {
    if (root.empty()) return;
    for (auto& kv : root) kv.second->flood_fill();
    std::vector<I3> keys;
    for (auto& kv : root) keys.push_back(kv.first);
    for (size_t n = 0; n + 1 < keys.size(); ++n) {
      I3 a = keys[n], b = keys[n + 1];
      if (a.x != b.x || a.y != b.y || b.z == a.z + CRES) continue;
      Sign as = root[a]->last_value_sign();
      Sign bs = root[b]->first_value_sign();
      if (as != Sign::Neg || bs != Sign::Neg) continue;
      I3 t = i3(a.x, a.y, a.z + CRES);
      while (t.z < b.z) {
        I3 k = root_key(t);
        auto node = C::empty(k);
        node->fill_with_sign(Sign::Neg);
        root[k] = std::move(node);
        t.z += CRES;
      }
    }
  }
  Sign sign_at(const I3& i) const {
    auto it = root.find(root_key(i));
    return it == root.end() ? Sign::Pos : it->second->sign_at(i);
  }
  // csg.rs:9-58
  void csg_union(std::unique_ptr<Root> other) {
    std::vector<I3> keys;
    for (auto& kv : root) keys.push_back(kv.first);
    for (auto& kv : other->root) keys.push_back(kv.first);
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    for (const I3& k : keys) {
      auto it = root.find(k);
      auto ot = other->root.find(k);
      if (ot == other->root.end()) continue;
      std::unique_ptr<C> n2 = std::move(ot->second);
      other->root.erase(ot);
      if (it != root.end())
        it->second->csg_union(std::move(n2));
      else
        root[k] = std::move(n2);
    }
  }
  void csg_subtract(std::unique_ptr<Root> other) {
    std::vector<I3> keys;
    for (auto& kv : other->root) keys.push_back(kv.first);
    for (const I3& k : keys) {
      auto it = root.find(k);
      if (it != root.end()) {
        auto ot = other->root.find(k);
        std::unique_ptr<C> n2 = std::move(ot->second);
        other->root.erase(ot);
        it->second->csg_subtract(std::move(n2));
      }
    }
  }
  void csg_intersect(std::unique_ptr<Root> other) {
    std::vector<I3> drop;
    for (auto& kv : root)
      if (!other->root.count(kv.first)) drop.push_back(kv.first);
    for (const I3& k : drop) root.erase(k);
    std::vector<I3> keys;
    for (auto& kv : root) keys.push_back(kv.first);
    for (const I3& k : keys) {
      auto ot = other->root.find(k);
      if (ot != other->root.end()) {
        std::unique_ptr<C> n2 = std::move(ot->second);
        other->root.erase(ot);
        root[k]->csg_intersect(std::move(n2));
      }
    }
  }
  void flip_signs() {
    for (auto& kv : root) kv.second->flip_signs();
  }
};

// voxel/volume/mod.rs:8 — dynamic_vdb!(f32, par 5, 4, 3)
using Leaf3 = Leaf<3>;
using Int4 = Internal<4, Leaf3>;
using Int5 = Internal<5, Int4>;
using Grid = Root<Int5>;

}  // namespace orc
