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
Schedule make_schedule(const std::vector<Box>& bricks, const std::vector<int>& brick_rank, int n_ranks,
                       const std::vector<KdNode>& tree, int order_mode, const float eye[3]);

}  // namespace aloha
