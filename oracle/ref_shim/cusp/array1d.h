/* Stand-in for cusp containers.  With LSREF_HOST_ONLY defined, "device"
 * arrays are host vectors so that host-only reference functions can run
 * without a GPU. */
#pragma once
#include <thrust/host_vector.h>
#include <thrust/device_vector.h>
namespace cusp {
struct host_memory {};
struct device_memory {};
template <class T, class M> struct array1d_sel { typedef thrust::host_vector<T> type; };
#ifndef LSREF_HOST_ONLY
template <class T> struct array1d_sel<T, device_memory> { typedef thrust::device_vector<T> type; };
#endif
template <class T, class M> using array1d = typename array1d_sel<T, M>::type;
template <class I, class T, class M> struct csr_matrix {};
template <class I, class T, class M> struct hyb_matrix {};
template <class I, class T, class M> struct ell_matrix {};
template <class I, class T, class M> struct coo_matrix {};
}
