// problem_host.h -- host-side problem model: Gset parsing with the
// reference's rules, integer adjacency, sweep colouring and the device
// site order.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace pticm {

struct HostProblem {
    int64_t n = 0;
    int64_t m = 0;               // edge count from the header / caller
    bool sparse = true;          // density < 10% (src/problem.cc:198)
    // adjacency in the reference's neighbour-list order, original indices
    std::vector<int64_t> row;    // n+1
    std::vector<int32_t> col;
    std::vector<int32_t> w;      // integer couplings J_ij
    std::vector<int32_t> h;      // integer linear terms (n)
    bool has_h = false;
    double char_scale = 0.0;     // max(mean w, var w) (src/problem.cc:244-245)
    double total_weight = 0.0;
    int32_t kmax = 0;            // max_i |h_i| + sum_j |J_ij|
    // sweep order: colour classes contiguous
    int32_t ncolors = 0;
    std::vector<int32_t> color_off;  // ncolors+1 (device indices)
    std::vector<int32_t> perm;       // device site -> original site
    std::vector<int32_t> iperm;      // original site -> device site
    // device adjacency (rows in device order, packed col<<8 | uint8(J))
    std::vector<int32_t> drow;
    std::vector<uint32_t> dadj;
    std::vector<int32_t> dh;

    void finalize();             // kmax, colouring, device layout
};

// Error codes follow pticm_status.  `msg` receives a description.
int parse_gset(const std::string& path, HostProblem& P, std::string& msg);
int problem_from_coo(int64_t n, int64_t m, const int32_t* src, const int32_t* dst, const double* w,
                     const double* h, HostProblem& P, std::string& msg);
int problem_from_dense(int64_t n, const double* J, const double* h, HostProblem& P, std::string& msg);

// beta_linspace of the reference (linear in beta, cumulative FP64 steps).
void beta_linspace(double* beta, double T0, double T1, uint64_t nt, bool inverse);

}  // namespace pticm
