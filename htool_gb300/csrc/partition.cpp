// Row partition of an H-matrix product over several GPUs.
//
// htool distributes the product by target rows: every MPI rank owns the
// rows of its clusters and computes them completely, with all-gathers of x
// before and of y after (include/htool/types/hmatrix.hpp:964-977, 1103).
// Here the cut points are chosen on the leaf list itself: a row c (cluster
// numbering) is a cut only if no leaf spans it, and the cuts balance the
// stored bytes each part reads.
#include "htgpu_internal.hpp"

#include <algorithm>
#include <vector>

namespace htgpu {

std::vector<int> partition_rows(int nleaves, const long long *leaves, int nr, int nparts) {
    require(nparts >= 1 && nr >= 0 && nleaves >= 0, "partition: bad sizes");
    // bytes per row start and the rows no leaf spans
    std::vector<long long> weight(nr + 1, 0);
    std::vector<int> span_end(nr + 1, 0); // largest end of the leaves starting at or before a row
    for (int l = 0; l < nleaves; l++) {
        const long long oi = leaves[3 * l], m = leaves[3 * l + 1], b = leaves[3 * l + 2];
        require(oi >= 0 && m >= 0 && oi + m <= nr && b >= 0, "partition: leaf outside the target rows");
        weight[oi] += b;
        span_end[oi] = std::max<int>(span_end[oi], (int)(oi + m));
    }
    std::vector<int> valid; // candidate cuts
    std::vector<long long> before;
    long long acc = 0;
    int reach     = 0;
    for (int c = 0; c <= nr; c++) {
        if (c >= reach) {
            valid.push_back(c);
            before.push_back(acc);
        }
        if (c < nr) {
            reach = std::max(reach, span_end[c]);
            acc += weight[c];
        }
    }
    std::vector<int> cuts(nparts + 1, 0);
    cuts[nparts] = nr;
    std::size_t k = 0;
    for (int p = 1; p < nparts; p++) {
        const double target = (double)acc * p / nparts;
        while (k + 1 < valid.size() && (double)before[k + 1] <= target)
            k++;
        // the nearer of the two candidates around the target
        std::size_t pick = k;
        if (k + 1 < valid.size() && (double)before[k + 1] - target < target - (double)before[k])
            pick = k + 1;
        cuts[p] = std::max(cuts[p - 1], valid[pick]);
    }
    return cuts;
}

} // namespace htgpu
