/* Stand-in for the dependency's cutil.h: constants and small vector macros. */
#pragma once
#include <cmath>
#include <cstdio>
#ifndef LARGENUM
#define LARGENUM 1000000000
#endif
#define CROSS_PRODUCT(a, b, c) { c[0] = a[1] * b[2] - a[2] * b[1]; c[1] = a[2] * b[0] - a[0] * b[2]; c[2] = a[0] * b[1] - a[1] * b[0]; }
#define DOT_PRODUCT(a, b) (a[0] * b[0] + a[1] * b[1] + a[2] * b[2])
#define DOT_PRODUCT2(a, b) (a[0] * b[0] + a[1] * b[1])
#define LENGTH(a) sqrt(DOT_PRODUCT(a, a))
#define LENGTH2(a) sqrt(DOT_PRODUCT2(a, a))
#define cudaSafeCall(x) do { (x); } while (0)
