// Grid clustering on the device (dbscan.cu).
#pragma once

#include "capi_internal.h"

namespace chaos {

// The reference's basin clustering (eps-connected components over flag != 0
// points, sign classes and canonical numbering); arrays are device pointers.
int dbscan_compat_device(Call& c, const double* avgPeaks, const double* avgIntervals, const int* flags, long long n,
                         double eps, int* labels);

// DBSCAN with scikit-learn semantics on the normalised features of a basin
// map, read from its per-point outputs: (amplitude, kept peak count, mean
// interval) min-max scaled over the points with flag != 0, the bounds taken
// from minmaxKeys (order keys: the three minima, then the three maxima).
// features (may be null) receives the n x 3 normalised matrix.
int dbscan_basins_device(Call& c, const BasinsOut& O, long long n, const unsigned long long* minmaxKeys, double eps,
                         int minPts, double* features, int* labels);

// DBSCAN with scikit-learn semantics on a row-major n x dims device matrix.
int dbscan_device(Call& c, const double* features, long long n, int dims, double eps, int minPts, const int* mask,
                  int* labels);

// Exclusive prefix sum of n ints / 64-bit ints (device arrays; in == out
// allowed); *total (host) receives the sum.
int exclusive_scan(Call& c, const int* in, int* out, long long n, int* total);
int exclusive_scan64(Call& c, const long long* in, long long* out, long long n, long long* total);

}  // namespace chaos
