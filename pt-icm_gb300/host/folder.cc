// folder.cc -- the reference's folder/CSV mode (src/main.cc:149-207) over the
// batch API: every (problem, restart) run of a folder in one persistent
// launch per ladder length, one CSV row per run.
#include <algorithm>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "pticm_gb300.hh"

namespace pticm {

namespace {

void check(int rc) {
    if (rc != PTICM_OK) throw std::runtime_error(std::string("pticm: ") + pticm_last_error());
}

// A value as an unmodified std::ostream writes it (six significant digits).
template <class T>
std::string plain(const T& v) {
    std::ostringstream o;
    o << v;
    return o.str();
}

// A vector as the reference's fstream overload writes it for a CSV cell
// (include/definitions.hh:22-33): quoted, "[a;b;c]".
template <class T>
std::string csv_list(const std::vector<T>& v) {
    std::string s = "\"[";
    for (size_t k = 0; k < v.size(); k++) s += (k ? ";" : "") + plain(v[k]);
    return s + "]\"";
}

struct Run {
    size_t file = 0, restart = 0;
    std::vector<double> beta;   // one chain's ladder (descending or ascending as chosen)
    double energy = 0.0, cut = 0.0;
    uint64_t flips = 0;
    std::vector<uint8_t> state;
    std::vector<double> pswap;
};

}  // namespace

size_t solve_folder(PTWorker& w, const std::string& folder, const std::string& csv_path, size_t restarts) {
    namespace fs = std::filesystem;
    std::vector<std::string> files;
    for (const auto& e : fs::directory_iterator(folder))
        if (e.is_regular_file()) files.push_back(e.path().string());
    // directory order is unspecified; sorted names make the rows reproducible
    std::sort(files.begin(), files.end());
    if (files.empty()) throw std::runtime_error("no problem files in " + folder);
    if (restarts == 0) throw std::runtime_error("--restarts must be at least 1");

    const Parameters P0 = w.params;
    std::vector<std::unique_ptr<Problem>> probs;
    std::vector<Run> runs;
    for (size_t f = 0; f < files.size(); f++) {
        probs.push_back(std::make_unique<Problem>(files[f], P0.seed, P0.burn_in));
        // the ladder of this problem (linspace, multihistogram or learned)
        w.params = P0;
        w.p = Problem(files[f], P0.seed, P0.burn_in);
        choose_ladder(w);
        for (size_t i = 0; i < restarts; i++) {
            Run r;
            r.file = f;
            r.restart = i;
            r.beta = w.beta_values;
            runs.push_back(std::move(r));
        }
    }
    w.params = P0;

    // one batch per ladder length (a batch shares nt and chains)
    std::map<size_t, std::vector<size_t>> by_nt;
    for (size_t k = 0; k < runs.size(); k++) by_nt[runs[k].beta.size()].push_back(k);
    for (const auto& [nt, members] : by_nt) {
        pticm_opts o;
        pticm_opts_default(&o);
        o.seed = P0.seed;
        o.nt = (uint32_t)nt;
        o.chains = P0.chains;
        o.sweeps = (uint32_t)P0.sweeps;
        o.icm = P0.icm ? 1 : 0;
        o.exchange = P0.exchange;
        o.best_per_phase = P0.best_per_phase;
        o.replicas_per_block = P0.replicas_per_block;
        o.block_threads = P0.block_threads;
        o.icm_algo = P0.icm_algo;
        std::vector<const pticm_problem*> ph;
        std::vector<double> ladders;
        for (size_t k : members) {
            ph.push_back(probs[runs[k].file]->handle());
            ladders.insert(ladders.end(), runs[k].beta.begin(), runs[k].beta.end());
        }
        pticm_batch* b = nullptr;
        check(pticm_batch_create(ph.data(), (uint32_t)ph.size(), &o, &b));
        std::unique_ptr<pticm_batch, void (*)(pticm_batch*)> hold(b, pticm_batch_destroy);
        check(pticm_batch_set_ladders(b, ladders.data(), (uint32_t)nt, -1));
        check(pticm_batch_init_states(b, P0.seed));
        if (ph.size() > 1 && P0.replicas_per_block == 0) check(pticm_batch_autotune(b, 20));
        check(pticm_batch_run(b, P0.pts, PTICM_PHASE_SWEEP | PTICM_PHASE_EXCHANGE | PTICM_PHASE_ICM));
        std::vector<double> E(ph.size());
        std::vector<uint64_t> fl(ph.size());
        check(pticm_batch_get_best(b, E.data(), fl.data()));
        const size_t R = nt * P0.chains;
        for (size_t j = 0; j < members.size(); j++) {
            Run& r = runs[members[j]];
            const Problem& p = *probs[r.file];
            r.energy = E[j];
            r.flips = fl[j];
            r.state.assign(p.vcount(), 0);
            check(pticm_batch_get_best_state(b, (uint32_t)j, r.state.data()));
            r.cut = p.maxcut(StateVector(r.state.begin(), r.state.end()));
            std::vector<uint64_t> att(R), suc(R);
            check(pticm_batch_get_swap_stats(b, (uint32_t)j, att.data(), suc.data()));
            r.pswap.assign(R, 0.0);
            for (size_t s = 0; s < R; s++) r.pswap[s] = att[s] ? (double)suc[s] / (double)att[s] : 0.0;
        }
    }

    std::ofstream file;
    if (!csv_path.empty()) {
        file.open(csv_path);
        if (!file) throw std::runtime_error("cannot write " + csv_path);
    }
    std::ostream& out = csv_path.empty() ? std::cout : file;
    out << "problem,iter,pts,replicas,tlist,pswap,icm,preprocess,burn_in,inverse,sweeps,ene,state,cut,flips\n";
    for (const Run& r : runs) {
        std::vector<double> tlist;   // the ladder of every chain (2 Nt values with two chains)
        for (uint32_t c = 0; c < P0.chains; c++) tlist.insert(tlist.end(), r.beta.begin(), r.beta.end());
        std::string bits;
        for (uint8_t s : r.state) bits += s ? '1' : '0';
        out << files[r.file] << "," << r.restart << "," << P0.pts << "," << r.beta.size() << "," << csv_list(tlist)
            << "," << csv_list(r.pswap) << "," << P0.icm << "," << P0.preprocess << "," << P0.burn_in << ","
            << P0.inverse << "," << P0.sweeps << "," << plain(r.energy) << ",\"" << bits << "\"," << plain(r.cut)
            << "," << r.flips << "\n";
    }
    out.flush();
    return runs.size();
}

}  // namespace pticm
