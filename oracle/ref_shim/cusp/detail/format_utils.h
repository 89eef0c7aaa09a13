/* offsets[i] = first position of index i in a sorted index array */
#pragma once
#include <thrust/binary_search.h>
#include <thrust/iterator/counting_iterator.h>
namespace cusp { namespace detail {
template <class A, class B> void indices_to_offsets(const A& idx, B& off) {
  thrust::lower_bound(idx.begin(), idx.end(), thrust::counting_iterator<int>(0),
                      thrust::counting_iterator<int>((int)off.size()), off.begin());
}
}}
