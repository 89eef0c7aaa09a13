// ls_partition.h -- graph partitioner (recursive graph bisection + greedy
// boundary refinement) for unstructured meshes.
#pragma once

namespace lsgb {
// npart[nv] <- part of each vertex, parts numbered 0..nparts-1; returns the
// number of parts used (min(nparts, nv)).  elems: ne x d1 vertex indices.
int partition_graph(int nv, const int* elems, int ne, int d1, int nparts, int* npart);
// number of mesh edges whose two vertices lie in different parts
long long edge_cut(int nv, const int* elems, int ne, int d1, const int* npart);
}  // namespace lsgb
