// problem_host.cc -- problem construction for the GPU engine.
//
// Parsing follows the reference's Problem(path) (src/problem.cc:183-247): a
// header "N M" ("N num_linear M" for .ising), one "u v [w]" line per edge, a
// missing weight meaning 1, lines of at most one character skipped, and
// 0-based vertices only when the path contains ".gset" or ".ising".  The
// reference stores sparse problems as neighbour lists in insertion order
// (duplicate lines become parallel edges, zero weights stay neighbours) and
// dense ones (density >= 10%) as an N x N matrix (later lines overwrite,
// zero entries are not neighbours); both behaviours are kept.
#include <algorithm>
#include <cmath>
#include <deque>
#include <fstream>
#include <limits>
#include <set>
#include <sstream>
#include <tuple>

#include "pticm.h"
#include "problem_host.h"

namespace pticm {

namespace {

bool as_small_int(double x, int32_t& out) {
    if (!std::isfinite(x) || x != std::floor(x) || x < -127.0 || x > 127.0) return false;
    out = (int32_t)x;
    return true;
}

// Build lists from (u, v, w) lines in push_back order.
void lists_from_lines(HostProblem& P, const std::vector<int64_t>& u, const std::vector<int64_t>& v,
                      const std::vector<int32_t>& w) {
    const int64_t n = P.n;
    P.row.assign(n + 1, 0);
    for (size_t k = 0; k < u.size(); k++) {
        P.row[u[k] + 1]++;
        P.row[v[k] + 1]++;
    }
    for (int64_t i = 0; i < n; i++) P.row[i + 1] += P.row[i];
    P.col.assign(P.row[n], 0);
    P.w.assign(P.row[n], 0);
    std::vector<int64_t> fill(P.row.begin(), P.row.end() - 1);
    for (size_t k = 0; k < u.size(); k++) {
        int64_t a = fill[u[k]]++;
        P.col[a] = (int32_t)v[k];
        P.w[a] = w[k];
        int64_t b = fill[v[k]]++;
        P.col[b] = (int32_t)u[k];
        P.w[b] = w[k];
    }
}

void lists_from_matrix(HostProblem& P, const std::vector<int32_t>& M) {
    const int64_t n = P.n;
    P.row.assign(n + 1, 0);
    P.col.clear();
    P.w.clear();
    for (int64_t i = 0; i < n; i++) {
        for (int64_t j = 0; j < n; j++)
            if (j != i && M[i * n + j] != 0) {
                P.col.push_back((int32_t)j);
                P.w.push_back(M[i * n + j]);
            }
        P.row[i + 1] = (int64_t)P.col.size();
    }
}

void set_scale(HostProblem& P, double sum, double sqsum, double M) {
    const double mean = sum / M;
    const double variance = sqsum / M - (sum / M * sum / M);
    P.char_scale = (mean >= variance) ? mean : variance;
}

}  // namespace

int parse_gset(const std::string& path, HostProblem& P, std::string& msg) {
    std::ifstream in(path);
    if (!in.is_open()) {
        msg = "cannot open " + path;
        return PTICM_ERR_IO;
    }
    const bool ising = path.find(".ising") != std::string::npos;
    const bool zero_based = ising || path.find(".gset") != std::string::npos;
    uint64_t N = 0, M = 0, num_linear = 0;
    if (ising) in >> N >> num_linear >> M;
    else in >> N >> M;
    if (!in || N == 0) {
        msg = "malformed header in " + path;
        return PTICM_ERR_IO;
    }
    if (N > (uint64_t)(1 << 24)) {
        msg = "more than 2^24 spins is not supported";
        return PTICM_ERR_UNSUPPORTED;
    }
    P = HostProblem();
    P.n = (int64_t)N;
    P.m = (int64_t)M;
    P.h.assign(N, 0);
    const uint64_t pairs = N * (N - 1) / 2;
    P.sparse = ((double)M / (double)pairs) < 0.1;
    const int64_t off = zero_based ? 0 : -1;
    std::vector<int64_t> us, vs;
    std::vector<int32_t> ws;
    std::vector<int32_t> dense;
    if (!P.sparse) dense.assign(N * N, 0);
    double sum = 0, sqsum = 0;
    uint64_t nlin = 0;
    std::string line;
    double w = 0.0;
    while (std::getline(in, line)) {
        if (line.size() <= 1) continue;
        std::istringstream ls(line);
        uint64_t u = 0, v = 0;
        if (nlin < num_linear) {
            double hv = 0;
            ls >> u >> hv;
            const int64_t ui = (int64_t)u + off;
            if (!ls.good() && !ls.eof()) {
                msg = "malformed linear term line: " + line;
                return PTICM_ERR_IO;
            }
            if (ui < 0 || ui >= (int64_t)N) {
                msg = "linear term index out of range: " + line;
                return PTICM_ERR_IO;
            }
            int32_t hi;
            if (!as_small_int(hv, hi)) {
                msg = "non-integer or out-of-range linear term: " + line;
                return PTICM_ERR_UNSUPPORTED;
            }
            P.h[ui] = hi;
            nlin++;
            continue;
        }
        ls >> u >> v;
        if (ls.fail()) {
            msg = "malformed edge line: " + line;
            return PTICM_ERR_IO;
        }
        if (ls.eof()) w = 1.0;
        else ls >> w;   // a failed read yields 0, as in the reference
        const int64_t ui = (int64_t)u + off, vi = (int64_t)v + off;
        if (ui < 0 || vi < 0 || ui >= (int64_t)N || vi >= (int64_t)N) {
            msg = "vertex index out of range: " + line;
            return PTICM_ERR_IO;
        }
        if (ui == vi) {
            msg = "self loop (the reference's dE algebra is wrong for it): " + line;
            return PTICM_ERR_UNSUPPORTED;
        }
        int32_t wi;
        if (!as_small_int(w, wi)) {
            msg = "coupling must be an integer in [-127, 127]: " + line;
            return PTICM_ERR_UNSUPPORTED;
        }
        sum += w;
        sqsum += w * w;
        if (P.sparse) {
            us.push_back(ui);
            vs.push_back(vi);
            ws.push_back(wi);
        } else {
            dense[ui * N + vi] = wi;
            dense[vi * N + ui] = wi;
        }
    }
    if (P.sparse) lists_from_lines(P, us, vs, ws);
    else lists_from_matrix(P, dense);
    set_scale(P, sum, sqsum, (double)M);
    P.finalize();
    return PTICM_OK;
}

int problem_from_coo(int64_t n, int64_t m, const int32_t* src, const int32_t* dst, const double* w,
                     const double* h, HostProblem& P, std::string& msg) {
    if (n <= 0 || m < 0 || (m > 0 && (!src || !dst || !w))) {
        msg = "invalid COO arguments";
        return PTICM_ERR_INVALID;
    }
    if (n > (int64_t)(1 << 24)) {
        msg = "more than 2^24 spins is not supported";
        return PTICM_ERR_UNSUPPORTED;
    }
    P = HostProblem();
    P.n = n;
    P.m = m;
    P.sparse = true;   // the COO constructor always builds lists
    P.h.assign(n, 0);
    std::vector<int64_t> us(m), vs(m);
    std::vector<int32_t> ws(m);
    double sum = 0, sq = 0;
    for (int64_t k = 0; k < m; k++) {
        if (src[k] < 0 || dst[k] < 0 || src[k] >= n || dst[k] >= n) {
            msg = "edge index out of range";
            return PTICM_ERR_INVALID;
        }
        if (src[k] == dst[k]) {
            msg = "self loops are not supported";
            return PTICM_ERR_UNSUPPORTED;
        }
        if (!as_small_int(w[k], ws[k])) {
            msg = "coupling must be an integer in [-127, 127]";
            return PTICM_ERR_UNSUPPORTED;
        }
        us[k] = src[k];
        vs[k] = dst[k];
        sum += w[k];
        sq += w[k] * w[k];
    }
    if (h)
        for (int64_t i = 0; i < n; i++)
            if (!as_small_int(h[i], P.h[i])) {
                msg = "linear term must be an integer in [-127, 127]";
                return PTICM_ERR_UNSUPPORTED;
            }
    lists_from_lines(P, us, vs, ws);
    if (m > 0) set_scale(P, sum, sq, (double)m);
    P.finalize();
    return PTICM_OK;
}

int problem_from_dense(int64_t n, const double* J, const double* h, HostProblem& P, std::string& msg) {
    if (n <= 0 || !J) {
        msg = "invalid dense arguments";
        return PTICM_ERR_INVALID;
    }
    if (n > 46340) {
        msg = "dense problems are limited to 46340 spins";
        return PTICM_ERR_UNSUPPORTED;
    }
    P = HostProblem();
    P.n = n;
    P.sparse = false;
    P.h.assign(n, 0);
    std::vector<int32_t> M(n * n, 0);
    double sum = 0, sq = 0;
    int64_t edges = 0;
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++) {
            if (i == j) continue;
            int32_t v;
            if (!as_small_int(J[i * n + j], v)) {
                msg = "coupling must be an integer in [-127, 127]";
                return PTICM_ERR_UNSUPPORTED;
            }
            M[i * n + j] = v;
            if (j > i && v != 0) {
                edges++;
                sum += v;
                sq += (double)v * v;
            }
        }
    P.m = edges;
    if (h)
        for (int64_t i = 0; i < n; i++)
            if (!as_small_int(h[i], P.h[i])) {
                msg = "linear term must be an integer in [-127, 127]";
                return PTICM_ERR_UNSUPPORTED;
            }
    lists_from_matrix(P, M);
    if (edges > 0) set_scale(P, sum, sq, (double)edges);
    P.finalize();
    return PTICM_OK;
}

// Colour the sites so that no two sites of a class interact: a BFS
// two-colouring when the graph is bipartite (checkerboard on even tori),
// otherwise greedy colouring in decreasing-degree order.
static int32_t colour_graph(const HostProblem& P, std::vector<int32_t>& colour) {
    const int64_t n = P.n;
    colour.assign(n, -1);
    bool bip = true;
    std::deque<int64_t> q;
    for (int64_t s = 0; s < n && bip; s++) {
        if (colour[s] >= 0) continue;
        colour[s] = 0;
        q.push_back(s);
        while (!q.empty() && bip) {
            const int64_t u = q.front();
            q.pop_front();
            for (int64_t a = P.row[u]; a < P.row[u + 1]; a++) {
                const int64_t v = P.col[a];
                if (colour[v] < 0) {
                    colour[v] = 1 - colour[u];
                    q.push_back(v);
                } else if (colour[v] == colour[u]) {
                    bip = false;
                    break;
                }
            }
        }
    }
    if (bip) {
        int32_t nc = 1;
        for (int64_t i = 0; i < n; i++) nc = std::max(nc, colour[i] + 1);
        return nc;
    }
    // greedy in decreasing-degree order (Welsh-Powell)
    std::vector<int64_t> order(n);
    for (int64_t i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        return (P.row[a + 1] - P.row[a]) > (P.row[b + 1] - P.row[b]);
    });
    colour.assign(n, -1);
    std::vector<int64_t> mark;
    int32_t nc = 0;
    for (int64_t u : order) {
        const int64_t deg = P.row[u + 1] - P.row[u];
        mark.assign(deg + 2, -1);
        for (int64_t a = P.row[u]; a < P.row[u + 1]; a++) {
            const int32_t c = colour[P.col[a]];
            if (c >= 0 && c <= deg) mark[c] = u;
        }
        int32_t c = 0;
        while (mark[c] == u) c++;
        colour[u] = c;
        nc = std::max(nc, c + 1);
    }
    // DSatur (Brelaz 1979): colour next the vertex whose neighbours already
    // use the most distinct colours (ties: higher degree, lower index);
    // usually fewer classes than greedy, and every class is one sweep phase.
    if (nc > 2 && nc <= 64) {
        std::vector<uint64_t> used(n, 0);
        std::vector<int32_t> sat(n, 0), dc(n, -1);
        // priority (saturation, degree, -index): vertices are ranked once by
        // (degree desc, index asc), and each saturation level keeps a bitmap
        // over ranks, so the next vertex is the lowest rank of the highest
        // non-empty level (lo[] bounds the first non-zero word of a level)
        std::vector<int64_t> ord(n), rank(n);
        for (int64_t i = 0; i < n; i++) ord[i] = i;
        std::stable_sort(ord.begin(), ord.end(), [&](int64_t x, int64_t y) {
            return (P.row[x + 1] - P.row[x]) > (P.row[y + 1] - P.row[y]);
        });
        for (int64_t r = 0; r < n; r++) rank[ord[r]] = r;
        const int64_t W = (n + 63) / 64;
        const int levels = nc + 1;
        std::vector<uint64_t> bits((size_t)levels * (size_t)W, 0);
        std::vector<int64_t> cnt(levels, 0), lo(levels, W);
        for (int64_t r = 0; r < n; r++) bits[(size_t)(r >> 6)] |= 1ull << (r & 63);
        cnt[0] = n;
        lo[0] = 0;
        int top = 0;
        int32_t nd = 0;
        bool fits = true;
        for (int64_t done = 0; done < n && fits; done++) {
            while (top > 0 && cnt[top] == 0) top--;
            uint64_t* lv = bits.data() + (size_t)top * (size_t)W;
            int64_t wi = lo[top];
            while (wi < W && lv[wi] == 0) wi++;
            if (wi == W) { fits = false; break; }   // (cannot happen: cnt[top] > 0)
            lo[top] = wi;
            const int64_t r0 = wi * 64 + __builtin_ctzll(lv[wi]);
            lv[wi] &= ~(1ull << (r0 & 63));
            cnt[top]--;
            const int64_t u = ord[r0];
            int32_t c = 0;
            while (c < 64 && (used[u] >> c) & 1ull) c++;
            if (c >= nc) { fits = false; break; }   // no better than greedy
            dc[u] = c;
            nd = std::max(nd, c + 1);
            for (int64_t a = P.row[u]; a < P.row[u + 1]; a++) {
                const int64_t v = P.col[a];
                if (dc[v] >= 0 || ((used[v] >> c) & 1ull)) continue;
                used[v] |= 1ull << c;
                const int sv = sat[v]++;
                if (sv + 1 >= levels) { fits = false; break; }
                const int64_t rv = rank[v], w = rv >> 6;
                const uint64_t bit = 1ull << (rv & 63);
                bits[(size_t)sv * (size_t)W + (size_t)w] &= ~bit;
                cnt[sv]--;
                bits[(size_t)(sv + 1) * (size_t)W + (size_t)w] |= bit;
                cnt[sv + 1]++;
                lo[sv + 1] = std::min(lo[sv + 1], w);
                top = std::max(top, sv + 1);
            }
        }
        if (fits && nd < nc) {
            colour = dc;
            nc = nd;
        }
    }
    return nc;
}

void HostProblem::finalize() {
    has_h = false;
    total_weight = 0.0;
    kmax = 0;
    for (int64_t i = 0; i < n; i++) {
        int64_t k = std::abs((int64_t)h[i]);
        if (h[i] != 0) has_h = true;
        for (int64_t a = row[i]; a < row[i + 1]; a++) {
            k += std::abs((int64_t)w[a]);
            total_weight += 0.5 * w[a];
        }
        kmax = (int32_t)std::max<int64_t>(kmax, k);
    }
    std::vector<int32_t> colour;
    ncolors = colour_graph(*this, colour);
    // device order: by colour, then by original index
    perm.resize(n);
    iperm.resize(n);
    color_off.assign(ncolors + 1, 0);
    for (int64_t i = 0; i < n; i++) color_off[colour[i] + 1]++;
    for (int32_t c = 0; c < ncolors; c++) color_off[c + 1] += color_off[c];
    std::vector<int32_t> fill(color_off.begin(), color_off.end() - 1);
    for (int64_t i = 0; i < n; i++) {
        const int32_t d = fill[colour[i]]++;
        perm[d] = (int32_t)i;
        iperm[i] = d;
    }
    drow.assign(n + 1, 0);
    dadj.clear();
    dadj.reserve(col.size());
    dh.assign(n, 0);
    for (int64_t d = 0; d < n; d++) {
        const int64_t i = perm[d];
        for (int64_t a = row[i]; a < row[i + 1]; a++)
            dadj.push_back(((uint32_t)iperm[col[a]] << 8) | ((uint32_t)(uint8_t)(int8_t)w[a]));
        drow[d + 1] = (int32_t)dadj.size();
        dh[d] = h[i];
    }
}

void beta_linspace(double* temps, double T0, double T1, uint64_t num_temp, bool inverse) {
    double step, curr;
    if (inverse) {
        step = T1 < T0 ? (T0 - T1) / (double)(num_temp - 1) : (T1 - T0) / (double)(num_temp - 1);
        curr = T1 < T0 ? T1 : T0;
    } else {
        step = T1 < T0 ? (1 / T1 - 1 / T0) / (double)(num_temp - 1) : (1 / T0 - 1 / T1) / (double)(num_temp - 1);
        curr = T1 < T0 ? 1 / T0 : 1 / T1;
    }
    for (uint64_t i = 0; i < num_temp; i++) {
        temps[i] = curr;
        curr += step;
    }
}

}  // namespace pticm
