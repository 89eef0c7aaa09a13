// ls_partition.cpp -- graph partitioner for unstructured meshes: recursive
// graph bisection on the vertex graph, then greedy boundary refinement.
//
// The reference partitions unstructured meshes with METIS_PartGraphKway
// (src/core3d/cuda/meshFIM3d.cu:354-421) into ceil(nv / metis_size) parts.
// METIS is not part of this project; this is a classical alternative that
// needs no geometry:
//   1. bisection of a connected vertex set by a level structure: a
//      pseudo-peripheral start vertex (repeated breadth-first searches from
//      the last vertex reached), then the first |A| vertices in breadth-first
//      order form one side, the rest the other (graph-growing bisection);
//   2. recursion until every part holds at most `target` vertices, with the
//      part counts split in proportion to the vertices;
//   3. refinement: boundary vertices move to the neighbouring part with
//      which they share the most edges when that lowers the edge cut and
//      keeps both parts within 3 % of their target size (a few greedy passes
//      in the spirit of Fiduccia-Mattheyses, without hill climbing).
// Disconnected sets are handled by breadth-first searches restarted from the
// lowest unvisited vertex.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "ls_partition.h"

namespace lsgb {

namespace {

struct Graph {
  std::vector<int> off, adj;
};

Graph build_graph(int nv, const int* elems, int ne, int d1) {
  std::vector<std::vector<int>> nb(nv);
  for (int e = 0; e < ne; ++e)
    for (int a = 0; a < d1; ++a)
      for (int b = 0; b < d1; ++b)
        if (a != b) nb[elems[(size_t)e * d1 + a]].push_back(elems[(size_t)e * d1 + b]);
  Graph g;
  g.off.assign(nv + 1, 0);
  for (int v = 0; v < nv; ++v) {
    auto& r = nb[v];
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    g.off[v + 1] = g.off[v] + (int)r.size();
  }
  g.adj.reserve(g.off[nv]);
  for (int v = 0; v < nv; ++v) g.adj.insert(g.adj.end(), nb[v].begin(), nb[v].end());
  return g;
}

// breadth-first order of the vertices in `set` (marked with `tag` in
// `owner`), starting at `start`, restarting at the lowest unvisited vertex
// of the set when a component is exhausted
void bfs_order(const Graph& g, const std::vector<int>& set, int start, const std::vector<int>& owner, int tag,
               std::vector<int>& seen, int stamp, std::vector<int>& order) {
  order.clear();
  size_t next_restart = 0;
  int s = start;
  while (true) {
    if (seen[s] != stamp) {
      seen[s] = stamp;
      size_t head = order.size();
      order.push_back(s);
      while (head < order.size()) {
        const int v = order[head++];
        for (int j = g.off[v]; j < g.off[v + 1]; ++j) {
          const int u = g.adj[j];
          if (owner[u] == tag && seen[u] != stamp) {
            seen[u] = stamp;
            order.push_back(u);
          }
        }
      }
    }
    if (order.size() == set.size()) break;
    while (next_restart < set.size() && seen[set[next_restart]] == stamp) ++next_restart;
    if (next_restart == set.size()) break;
    s = set[next_restart];
  }
}

}  // namespace

int partition_graph(int nv, const int* elems, int ne, int d1, int nparts, int* npart) {
  if (nv <= 0 || nparts <= 0) return 0;
  nparts = std::min(nparts, nv);
  const Graph g = build_graph(nv, elems, ne, d1);
  std::vector<int> owner(nv, 0), seen(nv, -1), order;
  int stamp = 0;
  // work list of (vertex set tag, first part id, number of parts)
  struct Job {
    std::vector<int> verts;
    int first, parts;
  };
  std::vector<Job> stack;
  Job root;
  root.verts.resize(nv);
  for (int v = 0; v < nv; ++v) root.verts[v] = v;
  root.first = 0;
  root.parts = nparts;
  stack.push_back(std::move(root));
  int next_tag = 1;
  while (!stack.empty()) {
    Job job = std::move(stack.back());
    stack.pop_back();
    if (job.parts <= 1 || job.verts.size() <= 1) {
      for (int v : job.verts) npart[v] = job.first;
      continue;
    }
    const int tag = next_tag++;
    for (int v : job.verts) owner[v] = tag;
    std::sort(job.verts.begin(), job.verts.end());
    // pseudo-peripheral start: two rounds of "start from the last vertex
    // reached"
    int start = job.verts[0];
    for (int round = 0; round < 2; ++round) {
      bfs_order(g, job.verts, start, owner, tag, seen, stamp++, order);
      start = order.back();
    }
    bfs_order(g, job.verts, start, owner, tag, seen, stamp++, order);
    const int left_parts = job.parts / 2;
    const size_t left_n = (size_t)std::llround((double)job.verts.size() * left_parts / job.parts);
    Job a, b;
    a.verts.assign(order.begin(), order.begin() + left_n);
    b.verts.assign(order.begin() + left_n, order.end());
    a.first = job.first;
    a.parts = left_parts;
    b.first = job.first + left_parts;
    b.parts = job.parts - left_parts;
    stack.push_back(std::move(a));
    stack.push_back(std::move(b));
  }
  // greedy boundary refinement
  std::vector<int> size(nparts, 0);
  for (int v = 0; v < nv; ++v) size[npart[v]]++;
  const double ideal = (double)nv / nparts;
  const int cap = (int)std::ceil(ideal * 1.03) + 1;
  const int floor_sz = std::max(1, (int)std::floor(ideal * 0.97) - 1);
  std::vector<int> cnt(nparts, 0), touched;
  for (int pass = 0; pass < 4; ++pass) {
    int moves = 0;
    for (int v = 0; v < nv; ++v) {
      const int pv = npart[v];
      touched.clear();
      for (int j = g.off[v]; j < g.off[v + 1]; ++j) {
        const int q = npart[g.adj[j]];
        if (cnt[q]++ == 0) touched.push_back(q);
      }
      int best = pv, best_gain = 0;
      for (int q : touched) {
        if (q == pv) continue;
        const int gain = cnt[q] - cnt[pv];
        if (gain > best_gain && size[q] + 1 <= cap && size[pv] - 1 >= floor_sz) {
          best = q;
          best_gain = gain;
        }
      }
      for (int q : touched) cnt[q] = 0;
      if (best != pv) {
        npart[v] = best;
        size[pv]--;
        size[best]++;
        moves++;
      }
    }
    if (moves == 0) break;
  }
  return nparts;
}

long long edge_cut(int nv, const int* elems, int ne, int d1, const int* npart) {
  const Graph g = build_graph(nv, elems, ne, d1);
  long long cut = 0;
  for (int v = 0; v < nv; ++v)
    for (int j = g.off[v]; j < g.off[v + 1]; ++j)
      if (npart[v] != npart[g.adj[j]]) ++cut;
  return cut / 2;
}

}  // namespace lsgb
