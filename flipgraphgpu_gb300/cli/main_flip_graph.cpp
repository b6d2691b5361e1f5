// flip_graph: drop-in replacement of the reference's executable of the same
// name (main_flip_graph.cu, FlipGraph in flip_graph.cu).  Same flags, same
// input format, same report table, same saved JSON files and file names; the
// walks run in libflipgraph (include/flipgraph.h).
//
// Additive flags (defaults reproduce the reference's behaviour):
//   --ring ZT|Z2|ZB       the reference picks the ring at compile time (ZT by default); ZB
//                         (integers with |c| <= 2, fast mode, naive starts) has no reference counterpart
//   --mode reference|fast reference = the reference's cuRAND stream, bit-exact trajectories
//   --max-launches N      stop after N launches (0: run forever, as the reference does)
//   --target-rank R       stop once a walk's best rank reaches R (0: off)
//   --time-budget S       stop after S seconds (0: off)
//   --gauss-probability P Gauss (XOR) reduction per step with probability P / max iterations (Z2;
//                         the reference defines SchemeZ2::tryReduceGauss but never calls it)
//   --ternary-sandwiching 1  ZT: the sandwiching move conjugates by random signed permutations
//                         (the reference's ternary sandwiching is empty)
//   --retry-cap N         bound on the loops the reference leaves unbounded (tryPlus's pair
//                         rejection, trySplitExisted, while (tryReduce())); a walk that exceeds it
//                         stops and a warning is printed (0: the library default, 2^20)
// Resize meta-operators (--resize-probability, default 0.2), sandwiching and
// basis-change moves run on both rings in the reference and philox modes and on
// the Z2 ring in the fast mode (grown factors of at most 56 entries there).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <numeric>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "common.h"
#include "scheme_io.h"

using namespace fgcli;
using Clock = std::chrono::high_resolution_clock;

namespace {

struct Options {
    int n1, n2, n3, schemes, maxIterations, plusIterations, logPeriod, seed;
    std::string path, inputPath, ring, mode;
    double expand, reduce, sandwiching, basis, resize, gauss, timeBudget;
    bool ternarySandwiching;
    int retryCap;
    long maxLaunches;
    int targetRank;
};

// Resizing, sandwiching and basis-change moves run in the list modes and in the fast mode on
// the Z2 ring; the Gauss reduction on the Z2 ring in every mode.
bool movesHere(const Options &o) { return o.mode != "fast" || o.ring == "Z2"; }  // sandwiching, basis changes
bool gaussHere(const Options &o) { return o.ring == "Z2"; }
bool resizeHere(const Options &o) { return o.mode != "fast" || o.ring == "Z2"; }

class FlipGraph {
public:
    FlipGraph(const Options &o) : o_(o), zt_(o.ring == "ZT"), zb_(o.ring == "ZB") {
        resizeOn_ = o.resize > 0 && resizeHere(o);
        n2bestRank_[key(o.n1, o.n2, o.n3)] = o.n1 * o.n2 * o.n3;
        known_ = knownRanks(zt_ || zb_);
    }
    ~FlipGraph() {
        if (h_) fg_destroy(h_);
    }

    bool initializeFromFile(std::istream &f) {  // flip_graph.cu:201-224
        int count = 0;
        f >> count;
        std::cout << "Start reading " << std::min(count, o_.schemes) << " schemes" << std::endl;
        std::vector<HostScheme> read;
        if (count <= 0) return false;
        for (int i = 0; i < count && i < o_.schemes; i++) {
            HostScheme s;
            s.zt = zt_;
            if (!s.read(f, false)) return false;
            while (s.tryReduce()) {
            }
            read.push_back(s);
        }
        std::cout << "Start copying " << std::min(count, o_.schemes) << " readed schemes" << std::endl;
        int cap = 4;
        for (const HostScheme &s : read) cap = std::max(cap, std::max(s.m, s.n[0] * s.n[1] * s.n[2]));
        create(cap);
        Records rec(o_.schemes, cap, zt_);
        for (int w = 0; w < o_.schemes; w++) {
            const HostScheme &s = read[w % read.size()];
            toRecords(s, rec.r, w, cap, true);
            if (w < (int)read.size() && !s.validate()) printf("not valid initialized scheme %d\n", w);
        }
        initRecords_ = std::move(rec);
        fromFile_ = true;
        return true;
    }

    void initializeNaive() {
        std::cout << "Start initializing with naive schemes" << std::endl;
        create(o_.n1 * o_.n2 * o_.n3);
        check(fg_init_naive(h_, o_.n1, o_.n2, o_.n3), "fg_init_naive");
    }

    void run() {  // flip_graph.cu:279-301
        initialize();
        auto startTime = Clock::now();
        auto t1 = Clock::now();
        std::vector<double> elapsedTimes;
        int stopped = 0;
        for (long iteration = 0;; iteration++) {
            fg_stats st;
            fg_status s = resizeOn_ ? fg_run_walks(h_, 1, &st) : fg_run(h_, 1, &st);
            if (s != FG_OK && s != FG_ERR_WALK) check(s, "fg_run");
            if (s == FG_ERR_WALK && st.walks_failed > stopped) {  // the reference would hang here
                stopped = st.walks_failed;
                std::cout << "Warning: " << stopped << " walk(s) stopped at a retry bound or a slot overflow "
                          << "(their schemes are kept; the other walks go on)" << std::endl;
            }
            auto t2 = Clock::now();
            elapsedTimes.push_back(std::chrono::duration_cast<std::chrono::milliseconds>(t2 - t1).count() / 1000.0);
            report(startTime, (int)iteration + 1, elapsedTimes);
            t1 = Clock::now();
            if (resizeOn_) {
                check(fg_resize(h_), "fg_resize");
                updateRanks((int)iteration, true);
            }
            if (o_.maxLaunches > 0 && iteration + 1 >= o_.maxLaunches) break;
            if (o_.targetRank > 0 && st.min_best_rank <= o_.targetRank) break;
            double total = std::chrono::duration_cast<std::chrono::milliseconds>(Clock::now() - startTime).count() / 1000.0;
            if (o_.timeBudget > 0 && total >= o_.timeBudget) break;
        }
    }

private:
    struct Records {
        std::vector<int32_t> n, m, list_size, flips, best_rank, best_m, status;
        std::vector<uint64_t> fac, sgn, best_fac, best_sgn;
        std::vector<uint8_t> valid, best_valid;
        std::vector<uint32_t> lists;
        std::vector<int64_t> rng_pos;
        fg_records r{};
        Records() = default;
        Records(int S, int cap, bool zt)
            : n(3 * S), m(S), list_size(3 * S), flips(S), best_rank(S), best_m(S), status(S),
              fac((size_t)S * 3 * cap), sgn(zt ? (size_t)S * 3 * cap : 0), best_fac((size_t)S * 3 * cap),
              best_sgn(zt ? (size_t)S * 3 * cap : 0), valid(zt ? (size_t)S * 3 * cap : 0),
              best_valid(zt ? (size_t)S * 3 * cap : 0), lists((size_t)S * 3 * FG_LIST_CAP), rng_pos(S) {
            bind();
        }
        Records(Records &&o) noexcept { *this = std::move(o); }
        Records &operator=(Records &&o) noexcept {
            n = std::move(o.n); m = std::move(o.m); list_size = std::move(o.list_size); flips = std::move(o.flips);
            best_rank = std::move(o.best_rank); best_m = std::move(o.best_m); status = std::move(o.status);
            fac = std::move(o.fac); sgn = std::move(o.sgn); best_fac = std::move(o.best_fac);
            best_sgn = std::move(o.best_sgn); valid = std::move(o.valid); best_valid = std::move(o.best_valid);
            lists = std::move(o.lists); rng_pos = std::move(o.rng_pos);
            bind();
            return *this;
        }
        void bind() {
            r = fg_records{n.data(), m.data(), fac.data(), sgn.empty() ? nullptr : sgn.data(),
                           valid.empty() ? nullptr : valid.data(), list_size.data(), lists.data(), flips.data(),
                           best_rank.data(), best_m.data(), best_fac.data(), best_sgn.empty() ? nullptr : best_sgn.data(),
                           best_valid.empty() ? nullptr : best_valid.data(), rng_pos.data(), status.data(),
                           /*best_n*/ nullptr, /*fac2*/ nullptr, /*best_fac2*/ nullptr};
        }
    };

    void create(int cap) {
        if (resizeOn_) cap = FG_MAX_RANK + 2;  // products reach the maximal rank
        cap_ = cap;
        fg_config c{};
        c.ring = zb_ ? FG_RING_ZB : (zt_ ? FG_RING_ZT : FG_RING_Z2);
        c.mode = o_.mode == "fast" ? FG_MODE_FAST : (o_.mode == "philox" ? FG_MODE_PHILOX_LISTS : FG_MODE_REFERENCE);
        c.walks = o_.schemes;
        c.cap = cap;
        c.seed = (uint64_t)(long long)o_.seed;  // curand_init takes the int seed widened
        c.iterations = o_.maxIterations;
        c.plus_iterations = o_.plusIterations;
        c.expand_p = o_.expand;
        c.reduce_p = o_.reduce;
        c.device = 0;
        c.resize_p = resizeOn_ ? o_.resize : 0.0;
        c.sandwich_p = movesHere(o_) ? o_.sandwiching : 0.0;
        c.basis_p = movesHere(o_) ? o_.basis : 0.0;
        c.gauss_p = gaussHere(o_) && !zt_ ? o_.gauss : 0.0;
        c.zt_sandwich = o_.ternarySandwiching ? 1 : 0;
        c.retry_cap = o_.retryCap;
        check(fg_create(&c, &h_), "fg_create");
    }

    // initializeSchemesKernel + updateRanks(0, false) (flip_graph.cu:190-199,249-277,510-518).
    void initialize() {
        std::cout << "Start main initialization" << std::endl;
        const int S = o_.schemes;
        std::vector<int32_t> n(3 * S), m(S);
        if (fromFile_) {
            for (int w = 0; w < S; w++) {
                initRecords_.flips[w] = 0;
                initRecords_.best_m[w] = initRecords_.m[w];
            }
            std::copy(initRecords_.fac.begin(), initRecords_.fac.end(), initRecords_.best_fac.begin());
            std::copy(initRecords_.sgn.begin(), initRecords_.sgn.end(), initRecords_.best_sgn.begin());
            std::copy(initRecords_.valid.begin(), initRecords_.valid.end(), initRecords_.best_valid.begin());
            n = initRecords_.n;
            m = initRecords_.m;
        } else {
            for (int w = 0; w < S; w++) {
                n[3 * w] = o_.n1; n[3 * w + 1] = o_.n2; n[3 * w + 2] = o_.n3;
                m[w] = o_.n1 * o_.n2 * o_.n3;
            }
        }
        keys_.resize(S);
        unkeys_.resize(S);
        for (int w = 0; w < S; w++) {
            keys_[w] = key(n[3 * w], n[3 * w + 1], n[3 * w + 2]);
            unkeys_[w] = key(n[3 * w], n[3 * w + 1], n[3 * w + 2], false);
            sortKeys_.push_back(key(n[3 * w], n[3 * w + 1], n[3 * w + 2], true, true));
            auto it = n2bestRank_.find(keys_[w]);
            if (it == n2bestRank_.end() || m[w] < it->second) n2bestRank_[keys_[w]] = m[w];
        }
        if (fromFile_) {
            for (int w = 0; w < S; w++) initRecords_.best_rank[w] = n2bestRank_[keys_[w]];
            check(fg_set_records(h_, &initRecords_.r), "fg_set_records");
            initRecords_ = Records();
        }
        std::cout << "Initialized" << std::endl;
    }

    // Keys of the walks' current sizes (they change while resizing).
    void refreshKeys() {
        const int S = o_.schemes;
        std::vector<int32_t> n(3 * S);
        check(fg_get_sizes(h_, n.data(), nullptr), "fg_get_sizes");
        for (int w = 0; w < S; w++) {
            keys_[w] = key(n[3 * w], n[3 * w + 1], n[3 * w + 2]);
            unkeys_[w] = key(n[3 * w], n[3 * w + 1], n[3 * w + 2], false);
            sortKeys_[w] = key(n[3 * w], n[3 * w + 1], n[3 * w + 2], true, true);
        }
    }

    // updateRanks (flip_graph.cu:249-277): the best rank per size; an improving walk's
    // current scheme becomes its best and is saved (with `save`).
    void updateRanks(int iteration, bool save) {
        const int S = o_.schemes;
        refreshKeys();
        std::vector<int32_t> m(S);
        check(fg_get_counters(h_, m.data(), nullptr, nullptr, nullptr, nullptr, nullptr), "fg_get_counters");
        std::unordered_map<std::string, int> n2bestIndex;
        std::vector<int32_t> copies, ranks(S);
        for (int i = 0; i < S; i++) {
            auto it = n2bestRank_.find(keys_[i]);
            if (it == n2bestRank_.end() || m[i] < it->second) {
                n2bestRank_[keys_[i]] = m[i];
                n2bestIndex[keys_[i]] = i;
                copies.push_back(i);
            }
        }
        check(fg_copy_to_best(h_, copies.data(), (int)copies.size()), "fg_copy_to_best");
        for (int i = 0; i < S; i++) ranks[i] = n2bestRank_[keys_[i]];
        check(fg_set_best_ranks(h_, ranks.data()), "fg_set_best_ranks");
        if (save) {
            for (auto pair : n2bestIndex) {
                HostScheme s = fetch(pair.second, false);
                std::string path = savePath(s, iteration, pair.second);
                s.saveJson(path);
                std::cout << "Best rank of " << pair.first << " was improved to " << ranks[pair.second]
                          << " (known: " << known_[pair.first] << ")! Scheme saved to \"" << path << "\"" << std::endl;
            }
            if (n2bestIndex.size()) std::cout << std::endl;
        }
    }

    HostScheme fetch(int walk, bool best) {
        return zb_ ? fetchSchemeZB(h_, walk, cap_, best) : fetchScheme(h_, walk, cap_, zt_, best);
    }

    std::string savePath(const HostScheme &s, int iteration, int runId) const {  // flip_graph.cu:386-399
        std::ostringstream ss;
        ss << o_.path << "/" << key(s.n[0], s.n[1], s.n[2]) << "_m" << s.m << "_c" << s.complexity() << "_iteration"
           << iteration << "_run" << runId << "_" << key(s.n[0], s.n[1], s.n[2], false) << "_" << o_.ring
           << ".json";
        return ss.str();
    }

    void report(Clock::time_point startTime, int iteration, const std::vector<double> &times) {  // flip_graph.cu:303-380
        const int S = o_.schemes, count = 3;
        if (resizeOn_) refreshKeys();
        std::vector<int32_t> m(S), bestRanks(S), bestM(S), flips(S);
        std::vector<uint8_t> valid(S);
        check(fg_get_counters(h_, m.data(), bestRanks.data(), bestM.data(), flips.data(), nullptr, valid.data()),
              "fg_get_counters");
        for (int w = 0; w < S; w++)
            if (!valid[w]) printf("invalid (%d) scheme (random walk)\n", w);
        double lastTime = times.back();
        double minTime = *std::min_element(times.begin(), times.end());
        double maxTime = *std::max_element(times.begin(), times.end());
        double meanTime = std::accumulate(times.begin(), times.end(), 0.0) / times.size();
        double elapsed = std::chrono::duration_cast<std::chrono::milliseconds>(Clock::now() - startTime).count() / 1000.0;

        // getSortedIndices (flip_graph.cu:401-415)
        std::unordered_map<std::string, std::vector<int>> n2indices;
        for (int i = 0; i < S; i++) n2indices[keys_[i]].push_back(i);
        int sortCount = std::min(count, S);
        for (auto pair : n2indices) {
            if ((int)pair.second.size() < sortCount) sortCount = (int)pair.second.size();
            auto &v = n2indices[pair.first];
            std::partial_sort(v.begin(), v.begin() + sortCount, v.end(),
                              [&](int a, int b) { return bestM[a] < bestM[b]; });
        }
        std::vector<std::string> keys;
        for (auto const &pair : n2indices) {
            const std::string &n = pair.first;
            int index = pair.second[0];
            keys.push_back(n);
            if (bestRanks[index] < n2bestRank_[n]) {
                HostScheme best = fetch(index, true);
                std::string path = savePath(best, iteration, index);
                best.saveJson(path);
                std::cout << "Best rank of " << n << " was improved from " << n2bestRank_[n] << " to "
                          << bestRanks[index] << " (known: " << known_[n] << ")! Scheme saved to \"" << path << "\""
                          << std::endl;
                n2bestRank_[n] = bestRanks[index];
            }
        }
        if (o_.logPeriod == 0 || iteration % o_.logPeriod == 0) {
            std::cout << std::endl << std::left;
            std::cout << "+--------------------------------------------------------------+" << std::endl;
            std::cout << "| Schemes            Iteration            Elapsed time         |" << std::endl;
            std::cout << "| " << std::right;
            std::cout << std::setw(7) << S << "            ";
            std::cout << std::setw(9) << iteration << "            ";
            std::cout << std::setw(12) << prettyTime(elapsed) << "         |" << std::endl;
            std::cout << "+--------+--------+--------+-------+------+------+-------------+" << std::endl;
            std::cout << "| run id |  size  |  real  | known | best | curr | flips count |" << std::endl;
            std::cout << "+--------+--------+--------+-------+------+------+-------------+" << std::endl;
            std::sort(keys.begin(), keys.end(), [&](const std::string &a, const std::string &b) {
                return sortKeys_[n2indices.at(a)[0]] < sortKeys_[n2indices.at(b)[0]];
            });
            for (const auto &k : keys) {
                const std::vector<int> &indices = n2indices[k];
                for (int i = 0; i < count && i < (int)indices.size(); i++) {
                    int w = indices[i];
                    std::cout << "| " << std::setw(6) << (w + 1) << " | " << std::setw(6) << k << " | " << std::setw(6)
                              << unkeys_[w] << " | " << std::setw(5) << known_[k] << " | " << std::setw(4)
                              << bestRanks[w] << " | " << std::setw(4) << m[w] << " | " << std::setw(11)
                              << prettyInt(flips[w]) << " |";
                    if (i == 0) {
                        std::cout << " total: " << indices.size();
                        if (bestRanks[indices[0]] <= known_[k])
                            std::cout << ", " << (bestRanks[indices[0]] == known_[k] ? "equal" : "BETTER!!!");
                    }
                    std::cout << std::endl;
                }
                std::cout << "+--------+--------+--------+-------+------+------+-------------+" << std::endl;
            }
            std::cout << "- iteration time (last / min / max / mean): " << prettyTime(lastTime) << " / "
                      << prettyTime(minTime) << " / " << prettyTime(maxTime) << " / " << prettyTime(meanTime)
                      << std::endl;
            std::cout << std::endl;
        }
    }

    Options o_;
    bool zt_, zb_;
    bool resizeOn_ = false;  // list mode and resize probability > 0
    fg_handle *h_ = nullptr;
    int cap_ = 0;
    bool fromFile_ = false;
    Records initRecords_;
    std::vector<std::string> keys_, unkeys_, sortKeys_;
    std::unordered_map<std::string, int> n2bestRank_, known_;
};

}  // namespace

int main(int argc, char *argv[]) {
    ArgParser parser("flip_graph", "Find fast matrix multiplication in parallel using CUDA");
    parser.add("-n1", ArgType::Natural, "INT", "number of first matrix rows");
    parser.add("-n2", ArgType::Natural, "INT", "number of first matrix columns and second matrix rows");
    parser.add("-n3", ArgType::Natural, "INT", "number of second matrix columns");
    parser.add("--schemes", ArgType::Natural, "INT", "number of schemes", "1024");
    parser.add("--max-iterations", ArgType::Natural, "INT", "number of flips per iterations", "10000");
    parser.add("--path", ArgType::String, "PATH", "path to save schemes", "schemes");
    parser.add("--input-path", ArgType::String, "PATH", "path to init schemes", "null");
    parser.add("--block-size", ArgType::Natural, "INT", "number of cuda threads (accepted; the library sizes its launches)", "32");
    parser.add("--expand-probability", ArgType::Real, "REAL", "expand edge probability (divided by max iterations)", "0.01");
    parser.add("--reduce-probability", ArgType::Real, "REAL", "reduce edge probability (divided by max iterations)", "0.0");
    parser.add("--sandwiching-probability", ArgType::Real, "REAL", "sandwiching edge probability (divided by max iterations)", "0.0");
    parser.add("--basis-probability", ArgType::Real, "REAL", "basis edge probability (divided by max iterations)", "0.0");
    parser.add("--resize-probability", ArgType::Real, "REAL", "project/extend edge probability", "0.2");
    parser.add("--plus-iterations", ArgType::Natural, "INT", "number of iterations of plus call", "8000");
    parser.add("--log-period", ArgType::Natural, "INT", "period of report printing", "0");
    parser.add("--seed", ArgType::Natural, "INT", "random seed", "0");
    parser.add("--ring", ArgType::String, "ZT|Z2|ZB", "coefficient ring (ZB: integers with |c| <= 2, fast mode)", "ZT");
    parser.add("--mode", ArgType::String, "MODE", "reference (bit-exact stream) | fast | philox", "reference");
    parser.add("--gauss-probability", ArgType::Real, "REAL",
               "Gauss (XOR) reduction probability (divided by max iterations; Z2)", "0.0");
    parser.add("--ternary-sandwiching", ArgType::Natural, "0|1",
               "ZT: sandwiching conjugates by random signed permutations (the reference's move is empty)", "0");
    parser.add("--retry-cap", ArgType::Natural, "INT",
               "bound on the reference's unbounded retry loops (0: the library default)", "0");
    parser.add("--max-launches", ArgType::Natural, "INT", "stop after this many launches (0: never)", "0");
    parser.add("--target-rank", ArgType::Natural, "INT", "stop when a best rank reaches this (0: off)", "0");
    parser.add("--time-budget", ArgType::Real, "REAL", "stop after this many seconds (0: off)", "0");
    if (!parser.parse(argc, argv)) return 0;

    Options o;
    o.n1 = std::stoi(parser.get("-n1"));
    o.n2 = std::stoi(parser.get("-n2"));
    o.n3 = std::stoi(parser.get("-n3"));
    o.schemes = std::stoi(parser.get("--schemes"));
    o.maxIterations = std::stoi(parser.get("--max-iterations"));
    o.path = parser.get("--path");
    o.inputPath = parser.get("--input-path");
    o.plusIterations = std::stoi(parser.get("--plus-iterations"));
    o.logPeriod = std::stoi(parser.get("--log-period"));
    o.seed = std::stoi(parser.get("--seed"));
    o.expand = std::stod(parser.get("--expand-probability"));
    o.reduce = std::stod(parser.get("--reduce-probability"));
    o.sandwiching = std::stod(parser.get("--sandwiching-probability"));
    o.basis = std::stod(parser.get("--basis-probability"));
    o.resize = std::stod(parser.get("--resize-probability"));
    o.gauss = std::stod(parser.get("--gauss-probability"));
    o.ternarySandwiching = parser.get("--ternary-sandwiching") == "1";
    o.retryCap = std::stoi(parser.get("--retry-cap"));
    o.ring = parser.get("--ring");
    o.mode = parser.get("--mode");
    o.maxLaunches = std::stol(parser.get("--max-launches"));
    o.targetRank = std::stoi(parser.get("--target-rank"));
    o.timeBudget = std::stod(parser.get("--time-budget"));
    if (o.ring != "ZT" && o.ring != "Z2" && o.ring != "ZB") {
        std::cerr << "unknown ring \"" << o.ring << "\"" << std::endl;
        return 0;
    }
    if (o.ring == "ZB") {  // integers with |c| <= 2: fast mode, naive starts
        if (o.mode != "fast") {
            std::cout << "Note: the ZB ring (|c| <= 2) runs in the fast mode" << std::endl;
            o.mode = "fast";
        }
        if (o.inputPath != "null") {
            std::cout << "Error: the ZB ring starts from the naive scheme (--input-path is not supported)" << std::endl;
            return -1;
        }
    }
    if (o.seed == 0) o.seed = (int)time(0);

    // Same checks, same operator precedence as main_flip_graph.cu:52-60.
    if ((o.inputPath == "null" && o.n1 * o.n2 > kMaxMatrixElements) || o.n2 * o.n3 > kMaxMatrixElements ||
        o.n1 * o.n3 > kMaxMatrixElements) {
        std::cout << "Error sizes, please increase MAX_MATRIX_ELEMENTS (now: " << kMaxMatrixElements << ")" << std::endl;
        return 0;
    }
    if (o.inputPath == "null" && o.n1 * o.n2 * o.n3 > kMaxRank) {
        std::cout << "Error sizes, please increase MAX_RANK (now: " << kMaxRank << ")" << std::endl;
        return 0;
    }

    std::cout << "Config:" << std::endl;
    std::cout << "- working ring: " << o.ring << std::endl;
    std::cout << "- max matrix elements: " << kMaxMatrixElements << std::endl;
    std::cout << "- max scheme rank: " << kMaxRank << std::endl;
    std::cout << "- min project size: 2" << std::endl;
    std::cout << "- max extension size: 16" << std::endl;
    std::cout << "- max flips pairs: " << FG_LIST_CAP << std::endl;
    std::cout << std::endl;
    std::cout << "Start flip graph algorithm" << std::endl;
    std::cout << "- n: " << o.n1 << " " << o.n2 << " " << o.n3 << std::endl;
    std::cout << "- schemes count: " << o.schemes << std::endl;
    std::cout << "- max iterations: " << o.maxIterations << std::endl;
    std::cout << "- plus iterations: " << o.plusIterations << std::endl;
    std::cout << "- path: " << o.path << std::endl;
    std::cout << "- block size: " << parser.get("--block-size") << std::endl;
    std::cout << "- probabilities:" << std::endl;
    std::cout << "  - expand: " << o.expand << std::endl;
    std::cout << "  - reduce: " << o.reduce << std::endl;
    std::cout << "  - sandwiching: " << o.sandwiching << std::endl;
    std::cout << "  - basis: " << o.basis << std::endl;
    std::cout << "  - resize: " << o.resize << std::endl;
    if (o.gauss > 0) std::cout << "  - gauss: " << o.gauss << std::endl;  // no reference counterpart
    std::cout << "- log period: " << o.logPeriod << std::endl;
    std::cout << "- seed: " << o.seed << std::endl;
    if (!movesHere(o) && (o.sandwiching > 0 || o.basis > 0))
        std::cout << "Note: sandwiching and basis-change moves are not available for the ZB ring; their "
                     "probabilities are treated as 0"
                  << std::endl;
    if (!resizeHere(o) && o.resize > 0)
        std::cout << "Note: resizing is not available for the ZB ring; its probability is treated as 0" << std::endl;
    if (o.gauss > 0 && o.ring != "Z2")
        std::cout << "Note: the Gauss reduction is defined for the Z2 ring only; its probability is treated as 0"
                  << std::endl;

    FlipGraph graph(o);
    if (o.inputPath != "null") {
        // The reference's text layout, or JSON saved by a run (a file or a directory of them).
        std::stringstream f;
        std::string error;
        if (!openSchemeInput(o.inputPath, TextLayout::FlipGraph, f, error)) {
            std::cout << error << std::endl;
            return -1;
        }
        bool ok = graph.initializeFromFile(f);
        if (!ok) return -1;
    } else {
        graph.initializeNaive();
    }
    try {
        graph.run();
        std::cout << "Success!" << std::endl;
    } catch (std::runtime_error &e) {
        std::cout << "Exception: " << e.what() << std::endl;
    }
    return 0;
}
