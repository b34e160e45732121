// libreplica.cc -- the reference's per-replica and per-pair interface over
// the C ABI: Replica (src/replica.cc), try_replica_exchange and its helpers
// (src/replica_exchange.cc), icm / xor_icm / bfs_icm (src/icm.cc), the
// initialisation of src/initialization.cc:5-100 and the gathers of
// src/mpi_utils.cc:77-226, for one worker that holds every replica.
//
// Random draws are the reference's: the host keeps Problem's std::mt19937_64
// and draws from it exactly where and as often as the reference does
// (Bernoulli initial spins, the sweep uniforms, the exchange log-uniforms and
// reshuffles, the ICM seed sample).  The per-site work -- sweeps, overlaps,
// cluster searches, field updates -- runs on the GPU.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>

#include "pticm_gb300.hh"

namespace pticm {

namespace {

void check(int rc) {
    if (rc != PTICM_OK) throw std::runtime_error(std::string("pticm: ") + pticm_last_error());
}

std::vector<uint8_t> bytes_of(const StateVector& s) { return std::vector<uint8_t>(s.begin(), s.end()); }

}  // namespace

// ------------------------------------------------------------------ Replica
Replica::Replica(Problem& p, double beta, const StateVector& init_state, const std::vector<double>& init_dE,
                 double energy, bool log_ene, size_t burn_in)
    : prob_(&p), beta_(beta), log_energy_(log_ene), burn_in_(burn_in) {
    (void)init_dE;   // the device computes the fields of init_state
    const std::vector<uint8_t> b = bytes_of(init_state);
    check(pticm_replica_create(p.handle(), beta, b.data(), &h_));
    if (log_ene) check(pticm_replica_set_logging(h_, 1, burn_in));
    energy_ = info().energy;
    if (energy != energy_) set_energy(energy);   // the reference keeps the caller's energy
}

Replica::Replica(const Replica& o)
    : prob_(o.prob_), energy_(o.energy_), beta_(o.beta_), log_energy_(o.log_energy_), sweeps_(o.sweeps_),
      burn_in_(o.burn_in_), ene_log_(o.ene_log_) {
    if (o.h_) check(pticm_replica_copy(o.h_, &h_));
}

Replica::Replica(Replica&& o) noexcept
    : h_(o.h_), prob_(o.prob_), energy_(o.energy_), beta_(o.beta_), log_energy_(o.log_energy_), sweeps_(o.sweeps_),
      burn_in_(o.burn_in_), state_fresh_(o.state_fresh_), dE_fresh_(o.dE_fresh_), best_fresh_(o.best_fresh_),
      state_(std::move(o.state_)), best_state_(std::move(o.best_state_)), dE_(std::move(o.dE_)),
      ene_log_(std::move(o.ene_log_)) {
    o.h_ = nullptr;
}

Replica& Replica::operator=(const Replica& o) {
    if (this != &o) {
        Replica tmp(o);
        *this = std::move(tmp);
    }
    return *this;
}

Replica& Replica::operator=(Replica&& o) noexcept {
    if (this != &o) {
        if (h_) pticm_replica_destroy(h_);
        h_ = o.h_;
        o.h_ = nullptr;
        prob_ = o.prob_;
        energy_ = o.energy_;
        beta_ = o.beta_;
        log_energy_ = o.log_energy_;
        sweeps_ = o.sweeps_;
        burn_in_ = o.burn_in_;
        state_fresh_ = o.state_fresh_;
        dE_fresh_ = o.dE_fresh_;
        best_fresh_ = o.best_fresh_;
        state_ = std::move(o.state_);
        best_state_ = std::move(o.best_state_);
        dE_ = std::move(o.dE_);
        ene_log_ = std::move(o.ene_log_);
    }
    return *this;
}

Replica::~Replica() {
    if (h_) pticm_replica_destroy(h_);
}

pticm_replica_info Replica::info() const {
    pticm_replica_info i{};
    if (!h_) throw std::runtime_error("pticm: the replica was never constructed");
    check(pticm_replica_get(h_, &i, nullptr, nullptr, nullptr));
    return i;
}

void Replica::set_energy(double e) {
    check(pticm_replica_set_energy(h_, e));
    energy_ = e;
}

const StateVector& Replica::get_state() const {
    if (!state_fresh_) {
        std::vector<uint8_t> b(prob_->vcount());
        check(pticm_replica_get(h_, nullptr, b.data(), nullptr, nullptr));
        state_.assign(b.begin(), b.end());
        state_fresh_ = true;
    }
    return state_;
}

StateVector& Replica::get_state() {
    static_cast<const Replica*>(this)->get_state();
    return state_;
}

uint64_t Replica::get_flips() const { return info().flips; }

void Replica::set_state(const StateVector& s) {
    const std::vector<uint8_t> b = bytes_of(s);
    check(pticm_replica_set_state(h_, b.data()));
    state_ = s;
    state_fresh_ = true;
    dE_fresh_ = false;
    energy_ = info().energy;
}

void Replica::set_dE(std::vector<double> dE) { (void)dE; }

void Replica::set_beta(double beta) {
    check(pticm_replica_set_beta(h_, beta));
    beta_ = beta;
}

std::vector<double>& Replica::get_dE() {
    if (!dE_fresh_) {
        dE_.resize(prob_->vcount());
        check(pticm_replica_get(h_, nullptr, nullptr, dE_.data(), nullptr));
        dE_fresh_ = true;
    }
    return dE_;
}

const StateVector& Replica::get_best_state() const {
    if (!best_fresh_) {
        std::vector<uint8_t> b(prob_->vcount());
        check(pticm_replica_get(h_, nullptr, nullptr, nullptr, b.data()));
        best_state_.assign(b.begin(), b.end());
        best_fresh_ = true;
    }
    return best_state_;
}

size_t Replica::get_best_sweep() const { return (size_t)info().best_sweep; }
double Replica::get_best_ene() const { return info().best_energy; }

void Replica::sweep(Problem& p) {
    const size_t n = p.vcount();
    // the sweep draws one uniform per uphill move (src/replica.cc:31-37):
    // draw n from a copy of the engine, then advance the engine itself by
    // exactly the number the GPU sweep used
    u_.resize(n);
    std::mt19937_64 g = p.get_rng();
    std::uniform_real_distribution<double> unif(0.0, 1.0);
    for (size_t i = 0; i < n; i++) u_[i] = unif(g);
    // the energy after every site is logged past the burn-in
    // (src/replica.cc:10-12: sweep_counter > burn_in)
    const bool logged = log_energy_ && sweeps_ > burn_in_;
    if (logged) elog_.resize(n);
    uint64_t used = 0;
    double e = 0.0;
    check(pticm_replica_sweep(h_, u_.data(), n, &used, &e, logged ? elog_.data() : nullptr));
    for (uint64_t k = 0; k < used; k++) p.rand_double();
    if (logged) ene_log_.insert(ene_log_.end(), elog_.begin(), elog_.end());
    sweeps_++;
    energy_ = e;
    state_fresh_ = dE_fresh_ = best_fresh_ = false;
}

// ------------------------------------------------------------------ worker
void read_problem(PTWorker& w, std::string problem_path) {
    w.p = Problem(problem_path, w.params.seed, w.params.burn_in);
    w.characteristic_scale = w.p.get_char_scale();
}

void initialize_replicas(PTWorker& w) {
    // src/initialization.cc:63-76: Bernoulli(1/2) spins from the problem's
    // engine, replica by replica, then the fields and energy
    std::bernoulli_distribution init_gen(0.5);
    w.replicas = std::vector<Replica>(w.loc_r);
    StateVector init_vector(w.p.vcount());
    for (size_t i = 0; i < w.loc_r; i++) {
        for (uint64_t j = 0; j < w.p.vcount(); j++) init_vector[j] = init_gen(w.p.get_rng());
        std::vector<double> dE(w.p.vcount(), 0);
        const double init_ene = w.p.calculate_dE(dE, init_vector);
        w.replicas[i] = Replica(w.p, w.beta_values_local[i], init_vector, dE, init_ene);
    }
}

void initialize_replica_exchanges(PTWorker& w) {
    // src/initialization.cc:77-100
    const size_t Nt = w.params.Nt;
    w.energy_values_global.assign(Nt * 2, 0.0);
    w.chain_1_exchange_order.assign(Nt - 1, 0);
    w.chain_2_exchange_order.assign(Nt - 1, 0);
    w.beta_indices.assign(Nt * 2, 0);
    w.swap_attempts.assign(Nt * 2, 0);
    w.swap_successes.assign(Nt * 2, 0);
    for (uint64_t i = 0; i + 1 < Nt; i++) {
        w.chain_1_exchange_order[i] = (uint32_t)i;
        w.chain_2_exchange_order[i] = (uint32_t)i;
    }
    for (uint64_t i = 0; i < Nt * 2; i++) w.beta_indices[i] = (uint32_t)i;
    w.exchange_index = 0;
    w.swaps = 0;
    std::shuffle(w.chain_1_exchange_order.begin(), w.chain_1_exchange_order.end(), w.p.get_rng());
    std::shuffle(w.chain_2_exchange_order.begin(), w.chain_2_exchange_order.end(), w.p.get_rng());
    w.energy_values_local.assign(w.loc_r, 0.0);
}

void gather_energy_values(PTWorker& w) {
    // src/mpi_utils.cc:77-101 with one worker
    std::copy(w.energy_values_local.begin(), w.energy_values_local.begin() + (long)w.loc_r,
              w.energy_values_global.begin());
}

Replica& get_replica(PTWorker& w, double beta, uint8_t chain) {
    // src/mpi_utils.cc:215-226
    for (size_t i = 0; i < w.loc_r; i++) {
        Replica& r = w.replicas[i];
        if (std::abs(beta - r.get_beta()) < 1e-10 && chain == w.chain_index_local[i]) return r;
    }
    throw std::runtime_error("pticm: no replica of chain " + std::to_string(chain) + " at beta " +
                             std::to_string(beta));
}

void do_replica_exchange_local(PTWorker& w, double beta_old, double beta_new, uint8_t chain_index) {
    // src/replica_exchange.cc:103-125: both replicas of the swap are local
    bool found = false;
    for (uint64_t j = 0; j < w.loc_r; j++) {
        if (std::abs(w.beta_values_local[j] - beta_new) < 1e-10 && w.chain_index_local[j] == chain_index) {
            w.beta_values_local[j] = beta_old;
            w.replicas[j].set_beta(beta_old);
            found = true;
        } else if (std::abs(w.beta_values_local[j] - beta_old) < 1e-10 && w.chain_index_local[j] == chain_index) {
            w.beta_values_local[j] = beta_new;
            w.replicas[j].set_beta(beta_new);
            found = true;
        }
    }
    if (!found) throw std::runtime_error("pticm: exchange found no replica at the swapped temperatures");
}

void check_for_replica_exchange(PTWorker& w) {
    // src/replica_exchange.cc:127-140 receives the manager's decision; the
    // manager is this worker, which applied it in try_replica_exchange
    (void)w;
}

void try_replica_exchange(PTWorker& w, uint8_t chain_index) {
    // src/replica_exchange.cc:5-100
    const uint64_t Nt = w.params.Nt;
    const uint64_t k = w.chain_1_exchange_order[w.exchange_index] + (chain_index ? Nt : 0);
    w.swap_attempts[k]++;
    const uint32_t r1 = w.beta_indices[k], r2 = w.beta_indices[k + 1];
    const double beta_low = w.beta_values[k], beta_high = w.beta_values[k + 1];
    const double dBeta = beta_low - beta_high;
    const double dE = w.energy_values_global[r1] - w.energy_values_global[r2];
    const double log_boltzmann = dBeta * dE;
    const double rndcomp = std::log(w.p.rand_double());
    if ((dE * dBeta) > 0 || rndcomp < log_boltzmann) {
        w.swap_successes[k]++;
        w.swaps++;
        if (w.params.verbosity >= 2)
            std::printf("\nSWAPPING temperatures %f <-> %f, dE = %f, in replicas %d and %d\n", beta_low, beta_high, dE,
                        0, 0);
        do_replica_exchange_local(w, beta_low, beta_high, chain_index);
        std::swap(w.beta_indices[k], w.beta_indices[k + 1]);
    }
    w.exchange_index++;
    if (w.exchange_index == Nt - 1) {
        w.exchange_index = 0;
        std::shuffle(w.chain_1_exchange_order.begin(), w.chain_1_exchange_order.end(), w.p.get_rng());
        std::shuffle(w.chain_2_exchange_order.begin(), w.chain_2_exchange_order.end(), w.p.get_rng());
    }
}

int64_t xor_icm(PTWorker& w, bool* state_1, bool* state_2) {
    // src/icm.cc:8-35: the overlap (and the global flip) on the GPU, the seed
    // drawn with std::sample from the differing sites in ascending order, as
    // the reference draws it
    const size_t n = w.p.vcount();
    std::vector<uint8_t> a(state_1, state_1 + n), b(state_2, state_2 + n);
    std::vector<int64_t> oneinds(n);
    uint64_t count = 0;
    check(pticm_problem_icm_overlap(w.p.handle(), a.data(), b.data(), &count, oneinds.data()));
    oneinds.resize(count);
    for (size_t j = 0; j < n; j++) state_1[j] = a[j] != 0;
    if (oneinds.empty()) return -1;
    std::vector<int64_t> seed_val(1);
    std::sample(oneinds.begin(), oneinds.end(), seed_val.begin(), 1, w.p.get_rng());
    return seed_val.front();
}

void bfs_icm(Problem& p, int64_t seed_val, bool* state_1, bool* state_2) {
    // src/icm.cc:37-72 on the GPU
    const size_t n = p.vcount();
    std::vector<uint8_t> a(state_1, state_1 + n), b(state_2, state_2 + n);
    check(pticm_problem_icm_cluster(p.handle(), seed_val, a.data(), b.data()));
    for (size_t j = 0; j < n; j++) {
        state_1[j] = a[j] != 0;
        state_2[j] = b[j] != 0;
    }
}

void icm(PTWorker& w, size_t target_replica) {
    // src/icm.cc:74-215, both replicas on this worker
    const double beta_val = w.beta_values[target_replica];
    const size_t n = w.p.vcount();
    std::unique_ptr<bool[]> state_1 = std::make_unique<bool[]>(n);
    std::unique_ptr<bool[]> state_2 = std::make_unique<bool[]>(n);
    Replica& r1 = get_replica(w, beta_val, 0);
    Replica& r2 = get_replica(w, beta_val, 1);
    const StateVector& s1 = r1.get_state();
    std::copy(s1.begin(), s1.end(), state_1.get());
    const StateVector& s2 = r2.get_state();
    std::copy(s2.begin(), s2.end(), state_2.get());
    const int64_t seed_val = xor_icm(w, state_1.get(), state_2.get());
    if (seed_val != -1) bfs_icm(w.p, seed_val, state_1.get(), state_2.get());
    // new states; the device recomputes their fields and energies
    r1.set_state(StateVector(state_1.get(), state_1.get() + n));
    r2.set_state(StateVector(state_2.get(), state_2.get() + n));
}

void check_icm(PTWorker& w) {
    // src/icm.cc:217-300 answers the manager's ICM messages; the manager is
    // this worker, which ran the move in icm()
    (void)w;
}

}  // namespace pticm
