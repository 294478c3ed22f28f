// Property check of the host visibility orders (aloha_gb300/csrc/order.cpp):
// on random grids of bricks (uneven cuts, some cells missing) and random eye
// points, with a random rank assignment (some leaving ranks without bricks),
//  * the brick order lists every brick once, and every pair is listed in an
//    order that some separating plane justifies (the first brick on the
//    eye's side of it, or the eye in the gap);
//  * each rank's bricks follow the brick order (the schedule's CSR lists);
//  * the rank order is the same property over the ranks' bounding boxes
//    when those are pairwise separable;
//  * a schedule from a freshly built cache equals the one from the kept
//    cache (the cache holds nothing that depends on the eye).
//
// Build: g++ -O2 -std=c++17 -I <csrc> -I <include> order_check.cpp <csrc>/order.cpp
// Prints one summary line; exit status 1 on any violation.
#include <cstdio>
#include <random>
#include <vector>

#include "order.h"

using aloha::Box;

namespace {

// Whether listing a before b is justified: some axis-aligned plane separates
// them with the eye not beyond b's near face (on a's side, or in the gap,
// where no ray from the eye can enter both).  Pairs that no plane separates
// carry no constraint here.
bool may_precede(const Box& a, const Box& b, const float eye[3]) {
  bool separable = false;
  for (int ax = 0; ax < 3; ++ax) {
    if (a.hi[ax] <= b.lo[ax]) {
      separable = true;
      if (eye[ax] <= b.lo[ax]) return true;
    }
    if (b.hi[ax] <= a.lo[ax]) {
      separable = true;
      if (eye[ax] >= b.hi[ax]) return true;
    }
  }
  return !separable;
}

bool check_order(const std::vector<Box>& boxes, const std::vector<int>& order, const float eye[3]) {
  const int n = (int)boxes.size();
  if ((int)order.size() != n) return false;
  std::vector<int> pos(n, -1);
  for (int k = 0; k < n; ++k) {
    if (order[k] < 0 || order[k] >= n || pos[order[k]] >= 0) return false;
    pos[order[k]] = k;
  }
  for (int k = 0; k < n; ++k)
    for (int l = k + 1; l < n; ++l)
      if (!may_precede(boxes[order[k]], boxes[order[l]], eye)) return false;
  return true;
}

}  // namespace

int main() {
  std::mt19937 rng(20240613u);
  std::uniform_real_distribution<float> U(0.f, 1.f);
  long cases = 0, bad = 0;
  for (int it = 0; it < 3000; ++it) {
    // uneven cuts per axis; each cell present with probability 0.85
    std::vector<float> cuts[3];
    for (int a = 0; a < 3; ++a) {
      const int m = 1 + (int)(U(rng) * 4);
      float x = 0.f;
      cuts[a].push_back(x);
      for (int k = 0; k < m; ++k) cuts[a].push_back(x += 16.f + (float)(int)(U(rng) * 100.f));
    }
    std::vector<Box> boxes;
    for (size_t z = 0; z + 1 < cuts[2].size(); ++z)
      for (size_t y = 0; y + 1 < cuts[1].size(); ++y)
        for (size_t x = 0; x + 1 < cuts[0].size(); ++x)
          if (boxes.empty() || U(rng) < 0.85f)
            boxes.push_back(Box{{cuts[0][x], cuts[1][y], cuts[2][z]}, {cuts[0][x + 1], cuts[1][y + 1], cuts[2][z + 1]}});
    const int nb = (int)boxes.size();
    const int R = 1 + (int)(U(rng) * nb);
    std::vector<int> br(nb);
    for (int b = 0; b < nb; ++b) br[b] = b < R ? b : (int)(U(rng) * R);
    if (it % 4 == 3 && R > 1)  // an explicit assignment may leave ranks without bricks
      for (int b = 0; b < nb; ++b) br[b] = (int)(U(rng) * (R / 2 + 1)) * 2 % R;
    const aloha::OrderCache cache = aloha::build_order_cache(boxes, br, R);
    // ranks' boxes are pairwise separable only when each rank holds one brick
    std::vector<int> per_rank(R, 0);
    for (int b = 0; b < nb; ++b) ++per_rank[br[b]];
    bool ranks_are_bricks = R == nb;
    for (int r = 0; r < R; ++r) ranks_are_bricks = ranks_are_bricks && per_rank[r] == 1;
    for (int e = 0; e < 12; ++e) {
      float eye[3];
      for (int a = 0; a < 3; ++a) eye[a] = (U(rng) * 3.f - 1.f) * cuts[a].back();
      if (e == 11)
        for (int a = 0; a < 3; ++a) eye[a] = cuts[a][cuts[a].size() / 2];  // on cut planes
      const std::vector<aloha::KdNode> no_tree;
      const aloha::Schedule s = aloha::make_schedule(boxes, br, R, no_tree, ALOHA_ORDER_FACES, eye, cache);
      std::vector<char> has(nb, 1);
      const std::vector<int> border = aloha::face_order(boxes, has, eye);
      ++cases;
      bool ok = check_order(boxes, border, eye);
      // CSR lists: each rank's bricks in brick order
      ok = ok && (int)s.rank_start.size() == R + 1 && s.rank_start[R] == nb;
      std::vector<int> pos(nb);
      for (int k = 0; k < nb; ++k) pos[border[k]] = k;
      for (int r = 0; ok && r < R; ++r)
        for (int k = s.rank_start[r]; k < s.rank_start[r + 1]; ++k) {
          ok = ok && br[s.rank_bricks[k]] == r;
          if (k > s.rank_start[r]) ok = ok && pos[s.rank_bricks[k - 1]] < pos[s.rank_bricks[k]];
        }
      // rank order: a permutation, and with one brick per rank the brick order
      std::vector<char> seen(R, 0);
      ok = ok && (int)s.rank_order.size() == R;
      for (int r : s.rank_order) ok = ok && r >= 0 && r < R && !seen[r] && (seen[r] = 1);
      if (ranks_are_bricks) {
        std::vector<Box> rb(R);
        for (int b = 0; b < nb; ++b) rb[br[b]] = boxes[b];
        ok = ok && check_order(rb, s.rank_order, eye);
      }
      // the one-shot form agrees with the cached one
      const aloha::Schedule s1 = aloha::make_schedule(boxes, br, R, no_tree, ALOHA_ORDER_FACES, eye,
                                                      aloha::build_order_cache(boxes, br, R));
      ok = ok && s1.rank_order == s.rank_order && s1.rank_bricks == s.rank_bricks;
      if (!ok && bad++ < 3) std::printf("violation: case %d, %d bricks, %d ranks\n", it, nb, R);
    }
  }
  std::printf("cases %ld violations %ld\n", cases, bad);
  return bad != 0;
}
