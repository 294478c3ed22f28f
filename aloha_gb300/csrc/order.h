// order.h -- virtual-rank partition and visibility order (host).
#pragma once

#include <vector>

#include "../../include/aloha.h"

namespace aloha {

struct Box {
  float lo[3], hi[3];
  static Box empty() { return Box{{1e30f, 1e30f, 1e30f}, {-1e30f, -1e30f, -1e30f}}; }
};

struct KdNode {
  int axis;
  float plane;
  int child1, child2;  // ~rank at leaves, INT_MAX when unset
};

struct Schedule {
  std::vector<int> rank_order;   // front to back
  std::vector<int> rank_start;   // CSR offsets by rank id
  std::vector<int> rank_bricks;  // each rank's bricks, front to back
};

bool partition_kd(const std::vector<Box>& boxes, int n_ranks, std::vector<int>& brick_rank,
                  std::vector<KdNode>& tree);
std::vector<int> kd_order(const std::vector<KdNode>& tree, const float eye[3]);
std::vector<int> face_order(const std::vector<Box>& item_bounds, const std::vector<char>& item_has_boxes,
                            const float eye[3]);

// The eye-independent part of face_order: which axis-aligned plane splits
// which set of items.  Built once per brick set and rank assignment; a view
// only walks it (near side first) and sorts the items of unsplittable sets by
// distance to its eye.
struct FaceTree {
  struct Node {
    int axis;       // < 0: a leaf holding items [first, second) of `items`
    float plane;
    int first, second;  // inner node: the subtrees below and above the plane
  };
  std::vector<Node> nodes;
  std::vector<int> items;
};
FaceTree build_face_tree(const std::vector<Box>& item_bounds, const std::vector<char>& item_has_boxes);
void face_order(const FaceTree& t, const std::vector<Box>& item_bounds, const std::vector<char>& item_has_boxes,
                const float eye[3], std::vector<int>& out);

// Everything make_schedule needs that does not depend on the eye.
struct OrderCache {
  FaceTree bricks;
  std::vector<char> brick_has;
  std::vector<Box> rank_bounds;
  std::vector<char> rank_has;
  FaceTree ranks;
};
OrderCache build_order_cache(const std::vector<Box>& bricks, const std::vector<int>& brick_rank, int n_ranks);
Schedule make_schedule(const std::vector<Box>& bricks, const std::vector<int>& brick_rank, int n_ranks,
                       const std::vector<KdNode>& tree, int order_mode, const float eye[3], const OrderCache& cache);

}  // namespace aloha
