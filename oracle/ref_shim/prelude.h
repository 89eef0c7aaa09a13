/* Pre-included (-include) before every reference translation unit. */
#pragma once
#include <cutil.h>
#include <thrust/host_vector.h>
#include <thrust/device_vector.h>
#include <thrust/sort.h>
#include <thrust/reduce.h>
#include <thrust/scan.h>
#include <thrust/unique.h>
#include <thrust/sequence.h>
#include <thrust/copy.h>
#include <thrust/fill.h>
#include <thrust/iterator/zip_iterator.h>
#include <iostream>
#include <algorithm>
#define cudaThreadSynchronize cudaDeviceSynchronize
