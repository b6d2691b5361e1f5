// complexity_minimizer: drop-in replacement of the reference's executable
// (main_complexity_minimizer.cu, ComplexityMinimizer in complexity_minimizer.cu).
// Same flags, input format, report and saved files; the flip walks run in
// libflipgraph.  Additive flag: --ring ZT|Z2 (the reference picks the ring at
// compile time, ZT by default).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "common.h"
#include "scheme_io.h"

using namespace fgcli;
using Clock = std::chrono::high_resolution_clock;

namespace {

class ComplexityMinimizer {
public:
    ComplexityMinimizer(int schemesCount, int maxIterations, const std::string &path, int seed, bool zt)
        : S_(schemesCount), maxIterations_(maxIterations), path_(path), seed_(seed), zt_(zt) {
        topCount_ = std::min(10, S_);
        for (int i = 0; i < S_; i++) indices_.push_back(i);
    }
    ~ComplexityMinimizer() {
        if (h_) fg_destroy(h_);
    }

    bool read(std::istream &f) {  // complexity_minimizer.cu:23-35
        int n1, n2, n3, m;
        f >> n1 >> n2 >> n3 >> m >> initialCount_;
        std::cout << "Start reading " << initialCount_ << " schemes (" << n1 << "x" << n2 << "x" << n3 << ": " << m
                  << ")" << std::endl;
        for (int i = 0; i < initialCount_; i++) {
            HostScheme s;
            s.zt = zt_;
            if (!s.readBody(f, n1, n2, n3, m, false)) return false;
            initial_.push_back(s);
        }
        std::cout << "Successfully read " << initialCount_ << " schemes" << std::endl;
        return true;
    }

    void minimize(int targetComplexity, int maxNoImprovements) {  // complexity_minimizer.cu:37-65
        initialize();
        auto startTime = Clock::now();
        std::vector<double> times;
        int noImprovements = 0;
        for (int iteration = 1; bestComplexity_ > targetComplexity; iteration++) {
            auto t1 = Clock::now();
            check(fg_minimize(h_, bestC_.data()), "fg_minimize");
            bool improved = updateBest(iteration);
            auto t2 = Clock::now();
            times.push_back(std::chrono::duration_cast<std::chrono::milliseconds>(t2 - t1).count() / 1000.0);
            report(startTime, iteration, times);
            if (improved) {
                noImprovements = 0;
            } else {
                noImprovements++;
                std::cout << "No improvements for " << noImprovements << " iterations" << std::endl;
                if (noImprovements >= maxNoImprovements) break;
            }
        }
    }

private:
    void initialize() {  // complexity_minimizer.cu:67-77,173-188
        bestComplexity_ = initial_[0].complexity();
        for (int i = 1; i < initialCount_; i++) bestComplexity_ = std::min(bestComplexity_, initial_[i].complexity());
        cap_ = 4;
        for (const HostScheme &s : initial_) cap_ = std::max(cap_, std::max(s.m, s.n[0] * s.n[1] * s.n[2]));
        fg_config c{};
        c.ring = zt_ ? FG_RING_ZT : FG_RING_Z2;
        c.mode = FG_MODE_REFERENCE;
        c.walks = S_;
        c.cap = cap_;
        c.seed = (uint64_t)(long long)seed_;
        c.iterations = maxIterations_;
        c.plus_iterations = 1 << 30;
        c.expand_p = 0.0;
        c.reduce_p = 0.0;
        check(fg_create(&c, &h_), "fg_create");
        allocRecords();
        for (int w = 0; w < S_; w++) {
            const HostScheme &s = initial_[w % initialCount_];
            if (w < initialCount_ && !s.validate()) printf("Invalid scheme %d\n", w);
            toRecords(s, rec_, w, cap_, true);
        }
        for (int w = 0; w < S_; w++) {
            rec_.best_m[w] = rec_.m[w];
            rec_.best_rank[w] = rec_.m[w];
            rec_.flips[w] = 0;
        }
        std::copy(fac_.begin(), fac_.end(), bfac_.begin());
        std::copy(sgn_.begin(), sgn_.end(), bsgn_.begin());
        std::copy(val_.begin(), val_.end(), bval_.begin());
        check(fg_set_records(h_, &rec_), "fg_set_records");
        bestC_.assign(S_, bestComplexity_);
    }

    void allocRecords() {
        const size_t nf = (size_t)S_ * 3 * cap_;
        n_.assign(3 * S_, 0); m_.assign(S_, 0); ls_.assign(3 * S_, 0); fl_.assign(S_, 0); br_.assign(S_, 0);
        bm_.assign(S_, 0); st_.assign(S_, 0); pos_.assign(S_, 0);
        fac_.assign(nf, 0); bfac_.assign(nf, 0); lists_.assign((size_t)S_ * 3 * FG_LIST_CAP, 0);
        if (zt_) { sgn_.assign(nf, 0); bsgn_.assign(nf, 0); val_.assign(nf, 0); bval_.assign(nf, 0); }
        rec_ = fg_records{n_.data(), m_.data(), fac_.data(), zt_ ? sgn_.data() : nullptr, zt_ ? val_.data() : nullptr,
                          ls_.data(), lists_.data(), fl_.data(), br_.data(), bm_.data(), bfac_.data(),
                          zt_ ? bsgn_.data() : nullptr, zt_ ? bval_.data() : nullptr, pos_.data(), st_.data(),
                          /*best_n*/ nullptr, /*fac2*/ nullptr, /*best_fac2*/ nullptr};
    }

    std::string savePath(const HostScheme &s, int iteration, int runId) const {  // complexity_minimizer.cu:136-149
        std::ostringstream ss;
        ss << path_ << "/" << key(s.n[0], s.n[1], s.n[2]) << "_m" << s.m << "_c" << s.complexity() << "_iteration"
           << iteration << "_run" << runId << "_" << key(s.n[0], s.n[1], s.n[2], false) << "_" << ringName(zt_)
           << ".json";
        return ss.str();
    }

    bool updateBest(int iteration) {  // complexity_minimizer.cu:86-99
        std::partial_sort(indices_.begin(), indices_.begin() + topCount_, indices_.end(),
                          [&](int a, int b) { return bestC_[a] < bestC_[b]; });
        int top = indices_[0];
        if (bestC_[top] >= bestComplexity_) return false;
        HostScheme best = fetchScheme(h_, top, cap_, zt_, true);
        std::string path = savePath(best, iteration, top);
        best.saveJson(path);
        std::cout << "Best complexity improved from " << bestComplexity_ << " to " << bestC_[top]
                  << "! Scheme saved to \"" << path << "\"" << std::endl;
        bestComplexity_ = bestC_[top];
        return true;
    }

    void report(Clock::time_point startTime, int iteration, const std::vector<double> &times) {  // :101-134
        double elapsed = std::chrono::duration_cast<std::chrono::milliseconds>(Clock::now() - startTime).count() / 1000.0;
        double lastTime = times.back();
        double minTime = *std::min_element(times.begin(), times.end());
        double maxTime = *std::max_element(times.begin(), times.end());
        double meanTime = std::accumulate(times.begin(), times.end(), 0.0) / times.size();
        check(fg_get_records(h_, &rec_), "fg_get_records");
        std::cout << "+-----------+-----------+--------+--------+--------+" << std::endl;
        std::cout << "|  elapsed  | iteration | run id |  best  |  curr  |" << std::endl;
        std::cout << "+-----------+-----------+--------+--------+--------+" << std::endl;
        for (int i = 0; i < topCount_ && i < S_; i++) {
            HostScheme s = fromRecords(rec_, indices_[i], cap_, zt_, false);
            std::cout << "| " << std::setw(9) << prettyTime(elapsed) << " | " << std::setw(9) << iteration << " | "
                      << std::setw(6) << (indices_[i] + 1) << " | " << std::setw(6) << bestC_[indices_[i]] << " | "
                      << std::setw(6) << s.complexity() << " |" << std::endl;
        }
        std::cout << "+-----------+-----------+--------+--------+--------+" << std::endl;
        std::cout << "- iteration time (last / min / max / mean): " << prettyTime(lastTime) << " / "
                  << prettyTime(minTime) << " / " << prettyTime(maxTime) << " / " << prettyTime(meanTime) << std::endl;
        std::cout << std::endl;
        // Walks restart from the global best (host rand(), complexity_minimizer.cu:130-133).
        int period = 1 + rand() % 10;
        HostScheme best = fromRecords(rec_, indices_[0], cap_, zt_, true);
        best.initFlips();
        bool changed = false;
        for (size_t i = 0; i < indices_.size(); i++)
            if (i % (iteration % period + 1) == 0) {
                toRecords(best, rec_, indices_[i], cap_, true);
                changed = true;
            }
        if (changed) check(fg_set_records(h_, &rec_), "fg_set_records");
    }

    int S_, maxIterations_;
    std::string path_;
    int seed_;
    bool zt_;
    int initialCount_ = 0, topCount_ = 10, cap_ = 0, bestComplexity_ = 0;
    fg_handle *h_ = nullptr;
    std::vector<HostScheme> initial_;
    std::vector<int> indices_;
    std::vector<int32_t> bestC_;
    std::vector<int32_t> n_, m_, ls_, fl_, br_, bm_, st_;
    std::vector<int64_t> pos_;
    std::vector<uint64_t> fac_, bfac_, sgn_, bsgn_;
    std::vector<uint8_t> val_, bval_;
    std::vector<uint32_t> lists_;
    fg_records rec_{};
};

}  // namespace

int main(int argc, char *argv[]) {
    ArgParser parser("flip_graph", "Find best complexity of the fast matrix multiplication scheme in parallel using CUDA");
    parser.add("--schemes", ArgType::Natural, "INT", "number of schemes", "1024");
    parser.add("--max-iterations", ArgType::Natural, "INT", "number of flips per iterations", "10000");
    parser.add("--path", ArgType::String, "PATH", "path to save schemes", "schemes");
    parser.add("--input-path", ArgType::String, "PATH", "path to init scheme(s)", "");
    parser.add("--block-size", ArgType::Natural, "INT", "number of cuda threads (accepted; the library sizes its launches)", "32");
    parser.add("--target-complexity", ArgType::Natural, "INT", "target complexity", "0");
    parser.add("--max-no-improvements", ArgType::Natural, "INT", "max iterations without improvements", "3");
    parser.add("--seed", ArgType::Natural, "INT", "random seed", "0");
    parser.add("--ring", ArgType::String, "ZT|Z2", "coefficient ring", "ZT");
    if (!parser.parse(argc, argv)) return 0;

    int schemesCount = std::stoi(parser.get("--schemes"));
    int maxIterations = std::stoi(parser.get("--max-iterations"));
    std::string path = parser.get("--path");
    std::string inputPath = parser.get("--input-path");
    std::string blockSize = parser.get("--block-size");
    int targetComplexity = std::stoi(parser.get("--target-complexity"));
    int maxNoImprovements = std::stoi(parser.get("--max-no-improvements"));
    int seed = std::stoi(parser.get("--seed"));
    std::string ring = parser.get("--ring");
    if (ring != "ZT" && ring != "Z2") {
        std::cerr << "unknown ring \"" << ring << "\"" << std::endl;
        return 0;
    }
    if (seed == 0) seed = (int)time(0);

    std::stringstream f;  // the reference's text layout, or JSON saved by a run
    std::string inputError;
    if (!openSchemeInput(inputPath, TextLayout::Minimizer, f, inputError)) {
        std::cout << inputError << std::endl;
        return -1;
    }
    std::cout << "Start complexity minimization algorithm" << std::endl;
    std::cout << "- schemes count: " << schemesCount << std::endl;
    std::cout << "- max iterations: " << maxIterations << std::endl;
    std::cout << "- path: " << path << std::endl;
    std::cout << "- block size: " << blockSize << std::endl;
    std::cout << "- target complexity: " << targetComplexity << std::endl;
    std::cout << "- max no improvements: " << maxNoImprovements << std::endl;
    std::cout << "- seed: " << seed << std::endl;

    ComplexityMinimizer minimizer(schemesCount, maxIterations, path, seed, ring == "ZT");
    bool result = minimizer.read(f);
    if (!result) {
        printf("Read invalid scheme\n");
        return -1;
    }
    try {
        minimizer.minimize(targetComplexity, maxNoImprovements);
        std::cout << "Success!" << std::endl;
    } catch (std::runtime_error &e) {
        std::cout << "Exception: " << e.what() << std::endl;
    }
    return 0;
}
