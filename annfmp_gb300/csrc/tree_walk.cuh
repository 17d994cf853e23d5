// tree_walk.cuh -- descent of the flat k-d tree (node arrays) with the top levels cached in shared
// memory; shared by the exact search, the row chain and the tensor-core leaf kernels.
#pragma once

#include "common.cuh"

namespace annf {

// ---------------------------------------------------------------------------------------------
// nodes: the top levels are cached in shared memory by the kernels that descend
// ---------------------------------------------------------------------------------------------
constexpr int kCacheLevels = 11;  // 2047 nodes

template <typename T>
struct NodeCache {
  int* axis;
  T* split;
  int n;  // cached nodes
  __device__ void fill(const TreeView<T>& tv, int levels = kCacheLevels) {
    const int lv = tv.depth < levels ? tv.depth : levels;
    n = (1 << lv) - 1;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      axis[i] = __ldg(tv.node_axis + i);
      split[i] = __ldg(tv.node_split + i);
    }
  }
  __device__ __forceinline__ void get(const TreeView<T>& tv, int node, int& ax, T& s) const {
    if (node < n) {
      ax = axis[node];
      s = split[node];
    } else {
      ax = __ldg(tv.node_axis + node);
      s = __ldg(tv.node_split + node);
    }
  }
  static size_t bytes(int depth, int levels = kCacheLevels) {
    const int lv = depth < levels ? depth : levels;
    const size_t m = (size_t)(1 << lv);
    return m * sizeof(int) + m * sizeof(T) + 32;
  }
  __device__ void carve(unsigned char*& p, int depth, int levels = kCacheLevels) {
    const int lv = depth < levels ? depth : levels;
    const int m = 1 << lv;
    axis = reinterpret_cast<int*>(p);
    split = reinterpret_cast<T*>(((uintptr_t)(axis + m) + 7) & ~uintptr_t(7));
    p = reinterpret_cast<unsigned char*>(((uintptr_t)(split + m) + 15) & ~uintptr_t(15));
  }
};

// leaf reached by descent: right when q[axis] - split >= 0 (kdtree.c:204)
template <typename T>
__device__ __forceinline__ int descend(const TreeView<T>& tv, const NodeCache<T>& nc, const T* q) {
  int node = 0;
  for (int l = 0; l < tv.depth; ++l) {
    int ax;
    T s;
    nc.get(tv, node, ax, s);
    node = (q[ax] >= s) ? 2 * node + 2 : 2 * node + 1;
  }
  return node - ((1 << tv.depth) - 1);
}

}  // namespace annf
