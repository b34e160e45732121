// mhist_host.h -- host side of the multihistogram ladder.
#pragma once
#include <cstdint>
#include <vector>

namespace pticm {

double partition_func(const std::vector<double>& logdos, double beta, double emin, double estep);
double acceptance_rate(const std::vector<double>& p1, const std::vector<double>& p2, double beta1, double beta2,
                       double estep, double emin);
uint32_t cae_walk(const std::vector<double>& logdos, double min_emin, double estep, double beta_start,
                  double beta_end, double step_size, double r, uint32_t num_temps, double* beta_out);

}  // namespace pticm
