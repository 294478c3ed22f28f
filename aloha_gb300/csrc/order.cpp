// order.cpp -- virtual-rank partition and per-view visibility order (host).
//
// partition_kd restates Partitioner::partitionKD (waikikiRenderer.cpp:150-270)
// and kd_order its computeCompositeOrder (281-316).  face_order is this
// library's default order: a separating-plane tree built from actual brick
// faces, which stays correct for bricks whose faces are not at the KD
// midplanes (the reference's midplane test can mis-order uneven bricks).
#include "order.h"

#include <algorithm>
#include <climits>
#include <utility>
#include <vector>

namespace aloha {

bool partition_kd(const std::vector<Box>& boxes, int n_ranks, std::vector<int>& brick_rank,
                  std::vector<KdNode>& tree) {
  struct Group {
    Box bounds;
    std::vector<int> ids;
    int node;
  };
  auto grow = [&](Box& b, int id) {
    for (int a = 0; a < 3; ++a) {
      b.lo[a] = std::min(b.lo[a], boxes[id].lo[a]);
      b.hi[a] = std::max(b.hi[a], boxes[id].hi[a]);
    }
  };
  const int n = (int)boxes.size();
  const size_t quota = (size_t)(n / n_ranks);
  Group root{Box::empty(), {}, 0};
  for (int i = 0; i < n; ++i) {
    grow(root.bounds, i);
    root.ids.push_back(i);
  }
  tree.assign(1, KdNode{0, 0.f, INT_MAX, INT_MAX});
  std::vector<Group> pending{root}, done;
  // With n_ranks <= bricks and bricks that tile space every split makes
  // progress; the cap turns a non-progressing split (which the reference
  // would repeat forever) into an error.
  size_t steps = 0;
  while (!pending.empty()) {
    if (++steps > 64 * boxes.size() + 64) return false;
    // the group with the most bricks (first one on ties)
    size_t pick = 0, most = 0;
    for (size_t k = 0; k < pending.size(); ++k)
      if (pending[k].ids.size() > most) {
        most = pending[k].ids.size();
        pick = k;
      }
    Group g = pending[pick];
    pending.erase(pending.begin() + (long)pick);
    if (g.ids.size() <= quota || done.size() == (size_t)n_ranks - 1) {
      const int rank = (int)done.size();
      tree[g.node].child1 = tree[g.node].child2 = ~rank;
      done.push_back(g);
      if (done.size() == (size_t)n_ranks) {
        for (const Group& rest : pending) done.back().ids.insert(done.back().ids.end(), rest.ids.begin(), rest.ids.end());
        pending.clear();
        break;
      }
      continue;
    }
    float ext[3];
    for (int a = 0; a < 3; ++a) ext[a] = g.bounds.hi[a] - g.bounds.lo[a];
    int axis = 0;
    if (ext[1] > ext[0] && ext[1] >= ext[2])
      axis = 1;
    else if (ext[2] > ext[0] && ext[2] >= ext[1])
      axis = 2;
    const float plane = g.bounds.lo[axis] + ext[axis] * 0.5f;
    Group lo{Box::empty(), {}, 0}, hi{Box::empty(), {}, 0};
    for (int id : g.ids) {
      Group& side = ((boxes[id].lo[axis] + boxes[id].hi[axis]) / 2.f < plane) ? lo : hi;
      grow(side.bounds, id);
      side.ids.push_back(id);
    }
    tree[g.node].axis = axis;
    tree[g.node].plane = plane;
    lo.node = (int)tree.size();
    tree[g.node].child1 = lo.node;
    tree.push_back(KdNode{0, 0.f, INT_MAX, INT_MAX});
    pending.push_back(lo);
    hi.node = (int)tree.size();
    tree[g.node].child2 = hi.node;
    tree.push_back(KdNode{0, 0.f, INT_MAX, INT_MAX});
    pending.push_back(hi);
  }
  brick_rank.assign(n, -1);
  for (size_t r = 0; r < done.size(); ++r)
    for (int id : done[r].ids) brick_rank[id] = (int)r;
  return true;
}

std::vector<int> kd_order(const std::vector<KdNode>& tree, const float eye[3]) {
  std::vector<int> order;
  if (tree.empty()) return order;
  std::vector<int> stack{0};
  int at = 0;
  while (!stack.empty()) {
    const KdNode& nd = tree[at];
    if (nd.child1 < 0 && nd.child2 < 0) {
      order.push_back(~nd.child1);
      at = stack.back();
      stack.pop_back();
    } else if (nd.child1 == INT_MAX) {
      at = stack.back();
      stack.pop_back();
    } else {
      const bool low_first = eye[nd.axis] < nd.plane;
      at = low_first ? nd.child1 : nd.child2;
      stack.push_back(low_first ? nd.child2 : nd.child1);
    }
  }
  return order;
}

namespace {

// The first axis-aligned plane (by axis, then position) that separates `items`
// into two non-empty sides, or false.
bool find_split(const std::vector<Box>& item_bounds, const std::vector<char>& item_has_boxes,
                const std::vector<int>& items, int& axis, float& plane, std::vector<int>& below,
                std::vector<int>& above) {
  if (items.size() <= 1) return false;
  for (int a = 0; a < 3; ++a) {
    std::vector<float> planes;
    for (int it : items)
      if (item_has_boxes[it]) {
        planes.push_back(item_bounds[it].lo[a]);
        planes.push_back(item_bounds[it].hi[a]);
      }
    std::sort(planes.begin(), planes.end());
    planes.erase(std::unique(planes.begin(), planes.end()), planes.end());
    for (float p : planes) {
      below.clear();
      above.clear();
      bool separates = true;
      for (int it : items) {
        if (!item_has_boxes[it] || item_bounds[it].hi[a] <= p)
          below.push_back(it);
        else if (item_bounds[it].lo[a] >= p)
          above.push_back(it);
        else {
          separates = false;
          break;
        }
      }
      if (separates && !below.empty() && !above.empty()) {
        axis = a;
        plane = p;
        return true;
      }
    }
  }
  return false;
}

}  // namespace

// Built with an explicit work list (a chain of bricks nests as deep as it is
// long): each job is an item set and the parent slot its node fills.
FaceTree build_face_tree(const std::vector<Box>& item_bounds, const std::vector<char>& item_has_boxes) {
  FaceTree t;
  struct Job {
    std::vector<int> items;
    int parent, side;  // side 0: the parent's `first` (below), 1: its `second` (above)
  };
  std::vector<Job> jobs;
  {
    std::vector<int> all(item_bounds.size());
    for (size_t i = 0; i < all.size(); ++i) all[i] = (int)i;
    if (!all.empty()) jobs.push_back(Job{std::move(all), -1, 0});
  }
  std::vector<int> below, above;
  while (!jobs.empty()) {
    Job j = std::move(jobs.back());
    jobs.pop_back();
    const int id = (int)t.nodes.size();
    if (j.parent >= 0) (j.side == 0 ? t.nodes[j.parent].first : t.nodes[j.parent].second) = id;
    int axis = 0;
    float plane = 0.f;
    if (find_split(item_bounds, item_has_boxes, j.items, axis, plane, below, above)) {
      t.nodes.push_back(FaceTree::Node{axis, plane, -1, -1});
      jobs.push_back(Job{above, id, 1});
      jobs.push_back(Job{below, id, 0});
    } else {
      // one item, or no plane separates them: ordered by distance per view
      t.nodes.push_back(FaceTree::Node{-1, 0.f, (int)t.items.size(), (int)(t.items.size() + j.items.size())});
      t.items.insert(t.items.end(), j.items.begin(), j.items.end());
    }
  }
  return t;
}

void face_order(const FaceTree& t, const std::vector<Box>& item_bounds, const std::vector<char>& item_has_boxes,
                const float eye[3], std::vector<int>& out) {
  out.clear();
  if (t.nodes.empty()) return;
  std::vector<int> stack(1, 0);
  std::vector<std::pair<float, int>> byd;
  while (!stack.empty()) {
    const FaceTree::Node& nd = t.nodes[stack.back()];
    stack.pop_back();
    if (nd.axis >= 0) {
      // the eye's side first (pushed last)
      const bool below_first = eye[nd.axis] < nd.plane;
      stack.push_back(below_first ? nd.second : nd.first);
      stack.push_back(below_first ? nd.first : nd.second);
      continue;
    }
    if (nd.second - nd.first <= 1) {
      out.insert(out.end(), t.items.begin() + nd.first, t.items.begin() + nd.second);
      continue;
    }
    byd.clear();
    for (int k = nd.first; k < nd.second; ++k) {
      const int it = t.items[k];
      float d2 = 0.f;
      for (int a = 0; a < 3; ++a) {
        const float c = item_has_boxes[it] ? (item_bounds[it].lo[a] + item_bounds[it].hi[a]) * 0.5f : eye[a];
        d2 += (c - eye[a]) * (c - eye[a]);
      }
      byd.push_back({d2, it});
    }
    std::stable_sort(byd.begin(), byd.end(), [](const std::pair<float, int>& l, const std::pair<float, int>& r) {
      return l.first < r.first;
    });
    for (auto& e : byd) out.push_back(e.second);
  }
}

std::vector<int> face_order(const std::vector<Box>& item_bounds, const std::vector<char>& item_has_boxes,
                            const float eye[3]) {
  std::vector<int> order;
  face_order(build_face_tree(item_bounds, item_has_boxes), item_bounds, item_has_boxes, eye, order);
  return order;
}

OrderCache build_order_cache(const std::vector<Box>& bricks, const std::vector<int>& brick_rank, int n_ranks) {
  OrderCache c;
  const int nb = (int)bricks.size();
  c.brick_has.assign(nb, 1);
  c.bricks = build_face_tree(bricks, c.brick_has);
  c.rank_bounds.assign(n_ranks, Box::empty());
  c.rank_has.assign(n_ranks, 0);
  for (int b = 0; b < nb; ++b) {
    const int r = brick_rank[b];
    if (r < 0 || r >= n_ranks) continue;
    c.rank_has[r] = 1;
    for (int a = 0; a < 3; ++a) {
      c.rank_bounds[r].lo[a] = std::min(c.rank_bounds[r].lo[a], bricks[b].lo[a]);
      c.rank_bounds[r].hi[a] = std::max(c.rank_bounds[r].hi[a], bricks[b].hi[a]);
    }
  }
  c.ranks = build_face_tree(c.rank_bounds, c.rank_has);
  return c;
}

Schedule make_schedule(const std::vector<Box>& bricks, const std::vector<int>& brick_rank, int n_ranks,
                       const std::vector<KdNode>& tree, int order_mode, const float eye[3], const OrderCache& cache) {
  const int nb = (int)bricks.size();
  Schedule s;
  // brick order: every brick is its own item
  std::vector<int> border;
  face_order(cache.bricks, bricks, cache.brick_has, eye, border);
  // rank order
  if (order_mode == ALOHA_ORDER_REFERENCE_KD && !tree.empty())
    s.rank_order = kd_order(tree, eye);
  else
    face_order(cache.ranks, cache.rank_bounds, cache.rank_has, eye, s.rank_order);
  // each rank's bricks in brick order (CSR by rank id)
  s.rank_start.assign(n_ranks + 1, 0);
  for (int b = 0; b < nb; ++b)
    if (brick_rank[b] >= 0 && brick_rank[b] < n_ranks) ++s.rank_start[brick_rank[b] + 1];
  for (int r = 0; r < n_ranks; ++r) s.rank_start[r + 1] += s.rank_start[r];
  s.rank_bricks.resize(s.rank_start[n_ranks]);
  std::vector<int> fill(s.rank_start.begin(), s.rank_start.end() - 1);
  for (int b : border)
    if (brick_rank[b] >= 0 && brick_rank[b] < n_ranks) s.rank_bricks[fill[brick_rank[b]]++] = b;
  return s;
}

}  // namespace aloha
