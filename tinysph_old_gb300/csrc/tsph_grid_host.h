// tsph_grid_host.h -- host-side cell-index tables (shared by the system API
// and the allocation-free binning entry point).
//
// The reference's cell index of a coordinate, (int)((x - x_0 + of)/kh)
// (src/SPH_find_pairs.h:64-65), is a monotone step function of the double x.
// cell_lower_bound() finds, by bisection over the ordered doubles and with
// the very same FP64 expression, the smallest double whose index is >= k;
// the device compares a coordinate's ordered bits against these bounds.
#pragma once

#include <climits>
#include <cstring>

#include "tsph_internal.cuh"

namespace tsph {

inline int ref_cell(double x, double x0, double of, double kh) {
    const double q = (x - x0 + of) / kh;
    if (!(q > -1e9)) return INT_MIN;
    if (!(q < 1e9)) return INT_MAX;
    return (int)q;
}

inline double from_ordered(long long o) {
    const long long b = o >= 0 ? o : (o ^ 0x7fffffffffffffffLL);
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

inline long long cell_lower_bound(int k, double x0, double of, double kh) {
    double span = 3.0;
    long long lo, hi;
    for (;;) {
        lo = ordered_bits(x0 - of + ((double)k - span) * kh);
        hi = ordered_bits(x0 - of + ((double)k + span) * kh);
        if (ref_cell(from_ordered(lo), x0, of, kh) < k && ref_cell(from_ordered(hi), x0, of, kh) >= k)
            break;
        span *= 2;
    }
    while ((unsigned long long)hi - (unsigned long long)lo > 1ull) {
        const long long mid = lo + (long long)(((unsigned long long)hi - (unsigned long long)lo) / 2ull);
        if (ref_cell(from_ordered(mid), x0, of, kh) >= k) hi = mid; else lo = mid;
    }
    return hi;
}

}  // namespace tsph
