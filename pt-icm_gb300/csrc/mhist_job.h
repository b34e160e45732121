// mhist_job.h -- one multihistogram fixed point of a batched solve.
#pragma once
#include <cstdint>

namespace pticm {

// Instance k of a batched solve: nt histogram rows starting at row0 of the
// per-row arrays (hoff, hlen, emin, beta, ln Z), nbins density-of-states
// bins starting at bin0 of the per-bin pools, bin i at min_emin + i*estep.
struct MhJob {
    int32_t nt;
    int32_t pad;
    int64_t row0;
    int64_t nbins;
    int64_t bin0;
    double min_emin;
    double estep;
    double logn;
};

}  // namespace pticm
