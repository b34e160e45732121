// pt_icm_main.cc -- the pt_icm command line (src/main.cc:15-209) on the GPU
// engine.  Same flags and defaults as the reference, the same report keys;
// `-g` is accepted as an alias of `-p` (the reference's README names it -g).
// Extra flags select GPU engine options.
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <iostream>
#include <stdexcept>
#include <string>

#include "pticm_gb300.hh"

namespace {

void usage() {
    std::printf(
        "Usage: pt_icm -p PROBLEM [options]\n"
        "  -s, --seed N                random seed (default: time)\n"
        "  -p, -g, --problem PATH      problem file (Gset; .gset/.ising names are 0-based)\n"
        "  -b, --burn_in N             burn-in steps (default 500)\n"
        "  --sweeps N                  sweeps per PT step (default 1)\n"
        "  -r, --replicas N            temperatures per chain (default 20)\n"
        "  --pts N                     PT steps (default 2000)\n"
        "  --preprocess-samples N      multihistogram samples (default 2000)\n"
        "  --preprocess-stepsize X     ladder walk step (default 0.1)\n"
        "  -T0, --temp0 X              first temperature (default 0.6)\n"
        "  -T1, --temp1 X              last temperature (default 2.8)\n"
        "  -i, --inverse               T0/T1 are inverse temperatures\n"
        "  --preprocess                multihistogram constant-acceptance ladder\n"
        "  --log                       print T,C,X,u,m per temperature from the steps after burn-in\n"
        "  --icm                       isoenergetic cluster moves\n"
        "  --verbose N                 verbosity\n"
        "GPU engine options:\n"
        "  --chains N                  replicas per temperature (default 2)\n"
        "  --exchange even-odd|reference   exchange attempt order (default even-odd)\n"
        "  --best-per-phase            check the best state after every colour class\n"
        "  --replicas-per-block N      replicas held by one thread block (default automatic)\n"
        "  --threads N                 threads per block (default automatic)\n"
        "  --icm-algo auto|bfs|union-find|label-prop\n"
        "  --sort-ladder               sort a --preprocess or learned ladder ascending (ICM on the coldest)\n"
        "  --learned-ladder FILE       constant-acceptance ladder from a trained surrogate network (no pilot\n"
        "                              run); checked by a short PT run, multihistogram ladder as fallback\n"
        "  --checkpoint FILE           write the PT state after the run (resumable)\n"
        "  --resume FILE               continue the run a checkpoint holds (same problem and options)\n"
        "Folder mode (the reference's unreachable src/main.cc:149-207), instead of --problem:\n"
        "  --folder DIR                run every problem file of DIR\n"
        "  --restarts N                runs per problem (default 1)\n"
        "  --csv FILE                  one row per run, the reference's columns (default: stdout)\n");
}

}  // namespace

int main(int argc, char** argv) {
    pticm::PTWorker w;
    pticm::Parameters& P = w.params;
    P.seed = (uint64_t)time(NULL);
    std::string problem_path, folder, csv;
    size_t restarts = 1;
    bool help = argc <= 1;
    try {
        for (int i = 1; i < argc; i++) {
            const std::string a = argv[i];
            auto next = [&]() -> std::string {
                if (i + 1 >= argc) throw std::runtime_error("missing value after " + a);
                return argv[++i];
            };
            if (a == "-h" || a == "--help") help = true;
            else if (a == "-s" || a == "--seed") P.seed = std::stoull(next());
            else if (a == "-p" || a == "-g" || a == "--problem") problem_path = next();
            else if (a == "-b" || a == "--burn_in") P.burn_in = std::stoull(next());
            else if (a == "--sweeps") P.sweeps = std::stoull(next());
            else if (a == "-r" || a == "--replicas") P.Nt = std::stoull(next());
            else if (a == "--pts") P.pts = std::stoull(next());
            else if (a == "--preprocess-samples") P.pre_samples = std::stoull(next());
            else if (a == "--preprocess-stepsize") P.pre_step = std::stod(next());
            else if (a == "-T0" || a == "--temp0") P.T0 = std::stod(next());
            else if (a == "-T1" || a == "--temp1") P.T1 = std::stod(next());
            else if (a == "-i" || a == "--inverse") P.inverse = true;
            else if (a == "--preprocess") P.preprocess = true;
            else if (a == "--log") P.log_data = true;
            else if (a == "--icm") P.icm = true;
            else if (a == "--verbose") P.verbosity = (uint32_t)std::stoul(next());
            else if (a == "--chains") P.chains = (uint32_t)std::stoul(next());
            else if (a == "--exchange") {
                const std::string v = next();
                if (v == "even-odd") P.exchange = 1;
                else if (v == "reference") P.exchange = 0;
                else throw std::runtime_error("--exchange takes even-odd or reference");
            } else if (a == "--best-per-phase") P.best_per_phase = 1;
            else if (a == "--replicas-per-block") P.replicas_per_block = (uint32_t)std::stoul(next());
            else if (a == "--threads") P.block_threads = (uint32_t)std::stoul(next());
            else if (a == "--icm-algo") {
                const std::string v = next();
                if (v == "auto") P.icm_algo = 0;
                else if (v == "bfs") P.icm_algo = 1;
                else if (v == "union-find") P.icm_algo = 2;
                else if (v == "label-prop") P.icm_algo = 3;
                else throw std::runtime_error("unknown --icm-algo " + v);
            } else if (a == "--sort-ladder") P.sort_ladder = true;
            else if (a == "--learned-ladder") P.learned_ladder = next();
            else if (a == "--resume") P.resume = next();
            else if (a == "--checkpoint") P.checkpoint = next();
            else if (a == "--folder") folder = next();
            else if (a == "--csv") csv = next();
            else if (a == "--restarts") restarts = std::stoull(next());
            else throw std::runtime_error("unknown argument " + a);
        }
        if (!help && problem_path.empty() && folder.empty()) throw std::runtime_error("--problem is required");
    } catch (const std::exception& e) {
        // the reference prints the error and the usage too, then carries on
        // with the empty path; here an argument error ends with status 1
        std::cout << e.what() << std::endl;
        usage();
        return 1;
    }
    if (help) {
        usage();
        return 0;
    }
    // print_args (src/main.cc:83-96)
    std::cout << "Seed: " << P.seed << std::endl;
    std::cout << "Replicas: " << P.Nt << std::endl;
    std::cout << "Sweeps: " << P.sweeps << std::endl;
    std::cout << "PT Steps: " << P.pts << std::endl;
    std::cout << "Burn-in: " << P.burn_in << std::endl;
    std::cout << "T0: " << P.T0 << std::endl;
    std::cout << "T1: " << P.T1 << std::endl;
    std::cout << "Inverse: " << P.inverse << std::endl;
    std::cout << "Preprocess: " << P.preprocess << std::endl;
    std::cout << "Log Data: " << P.log_data << std::endl;
    std::cout << "ICM: " << P.icm << std::endl;
    std::cout << "Verbosity: " << P.verbosity << std::endl;
    std::cout << (folder.empty() ? problem_path : folder) << std::endl;
    if (!folder.empty()) {
        try {
            const size_t rows = pticm::solve_folder(w, folder, csv, restarts);
            if (!csv.empty()) std::cout << rows << " runs written to " << csv << std::endl;
        } catch (const std::exception& e) {
            std::fprintf(stderr, "pt_icm: %s\n", e.what());
            return 1;
        }
        return 0;
    }
    try {
        double best_ene = 0;
        size_t flips = 0;
        pticm::StateVector best_state;
        pticm::solve(w, problem_path, best_ene, flips, best_state);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "pt_icm: %s\n", e.what());
        return 1;
    }
    return 0;
}
