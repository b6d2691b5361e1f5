// additions_reducer: drop-in replacement of the reference's executable
// (main_additions_reducer.cu, SchemeAdditionsReducer in
// scheme_additions_reducer.cu).  Same flags, checks, report and saved JSON;
// the reducers run in libflipgraph (fg_reducer_*).
//
// Additive flag: --z2-input 1 reads the scheme without the integer validity
// check, so schemes that are valid only modulo 2 can be reduced (the
// reference rejects them, scheme_additions_reducer.cu:48-51).
// --max-flips > 0: before every iteration after the first, schemes 1.. are
// flipped copies of the input (fg_reducer_flip) and the best reducer is chosen
// by its total over U, V and W (scheme_additions_reducer.cu:172-182,296-339).
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
#include <vector>

#include "common.h"
#include "scheme_io.h"

using namespace fgcli;
using Clock = std::chrono::high_resolution_clock;

namespace {

// Host replay of one component's AdditionsReducer: naive expressions, then
// the fresh variables applied in order (additions_reducer.cuh:67-86,218-301).
struct Expressions {
    std::vector<std::vector<int>> e;
    std::vector<std::pair<int, int>> vars;
    int real = 0;

    static int search(const std::vector<int> &x, int value, int start) {
        int lo = start, hi = (int)x.size() - 1, va = std::abs(value);
        while (lo <= hi) {
            int mid = lo + (hi - lo) / 2, ma = std::abs(x[mid]);
            if (ma < va) lo = mid + 1;
            else if (ma > va) hi = mid - 1;
            else return mid;
        }
        return -1;
    }

    void replace(int pi, int pj) {
        int var = real + (int)vars.size() + 1;
        for (auto &x : e) {
            if (x.size() < 2) continue;
            int i = search(x, pi, 0);
            if (i == -1) continue;
            int j = search(x, pj, i + 1);
            if (j == -1) continue;
            int v;
            if (x[i] == pi && x[j] == pj) v = var;
            else if (x[i] == -pi && x[j] == -pj) v = -var;
            else continue;
            std::vector<int> y;
            for (int q = 0; q < (int)x.size(); q++)
                if (q != i && q != j) y.push_back(x[q]);
            y.push_back(v);
            x.swap(y);
        }
        vars.push_back({pi, pj});
    }

    // AdditionsReducer::write (additions_reducer.cuh:304-347).
    void write(std::ostream &os, const std::string &name, const std::string &indent) const {
        os << indent << "\"" << name << "_fresh\": [" << std::endl;
        for (size_t i = 0; i < vars.size(); i++) {
            int a = vars[i].first, b = vars[i].second;
            os << indent << indent << "[{\"index\": " << std::abs(a) - 1 << ", \"value\": " << (a > 0 ? 1 : -1)
               << "}, {\"index\": " << std::abs(b) - 1 << ", \"value\": " << (b > 0 ? 1 : -1) << "}]";
            if (i + 1 < vars.size()) os << ",";
            os << std::endl;
        }
        os << indent << "]," << std::endl;
        os << indent << "\"" << name << "\": [" << std::endl;
        for (size_t i = 0; i < e.size(); i++) {
            os << indent << indent << "[";
            for (size_t j = 0; j < e[i].size(); j++) {
                os << "{\"index\": " << std::abs(e[i][j]) - 1 << ", \"value\": " << (e[i][j] > 0 ? 1 : -1) << "}";
                if (j + 1 < e[i].size()) os << ", ";
            }
            os << "]";
            if (i + 1 < e.size()) os << ",";
            os << std::endl;
        }
        os << indent << "]";
    }
};

// Per component state of one reducer as the host sees it.
struct ReducerView {
    int additions = 0, fresh = 0, naive = 0, mode = 0;
    float scale = 0;
    std::vector<int32_t> vars;  // [500][2]
};

std::string modeName(int mode, float scale) {  // additions_reducer.cuh:183-204
    switch (mode) {
        case 0: return "g";
        case 1: return "ga";
        case 2: return "gr" + std::to_string(int(scale * 100));
        case 3: return "gi" + std::to_string(int(scale * 100));
        case 4: return "wr";
        case 6: return "rnd";
    }
    return "mix";
}

class SchemeAdditionsReducer {
public:
    SchemeAdditionsReducer(int count, int schemesCount, int maxFlips, int seed, const std::string &out, bool z2input)
        : count_(count), schemesCount_(schemesCount), maxFlips_(maxFlips), seed_(seed), out_(out), z2input_(z2input) {
        topCount_ = std::min(10, count);
        for (int c = 0; c < 3; c++)
            for (int j = 0; j < count; j++) indices_[c].push_back(j);
        std::cout << "Start memory allocating" << std::endl;
    }
    ~SchemeAdditionsReducer() {
        if (h_) fg_reducer_destroy(h_);
    }

    bool read(std::istream &f) {  // scheme_additions_reducer.cu:29-90
        f >> n1_ >> n2_ >> n3_ >> m_;
        std::cout << "Start reading scheme " << n1_ << "x" << n2_ << "x" << n3_ << " with " << m_ << " multiplications"
                  << std::endl;
        if (m_ > kMaxRank) {
            std::cout << "Error: expressions count for U (" << m_ << ") too big for compiled configuration (" << kMaxRank
                      << ")" << std::endl;
            return false;
        }
        if (m_ > kMaxRank) {
            std::cout << "Error: expressions count for V (" << m_ << ") too big for compiled configuration (" << kMaxRank
                      << ")" << std::endl;
            return false;
        }
        if (n3_ * n1_ > kMaxMatrixElements) {
            std::cout << "Error: expressions count for W (" << (n3_ * n1_) << ") too big for compiled configuration ("
                      << kMaxMatrixElements << ")" << std::endl;
            return false;
        }
        scheme_.zt = true;
        if (!scheme_.readBody(f, n1_, n2_, n3_, m_, !z2input_)) {
            std::cout << "Error: readed scheme is invalid" << std::endl;
            return false;
        }
        // Real-variable and subexpression limits (scheme_additions_reducer.cu:53-88), including the
        // reference's comparison of realU against the W limit.
        int realU = maxReal(0), realV = maxReal(1), realW = maxReal(2);
        if (realU > kMaxMatrixElements / 2) {
            std::cout << "Error: real variables for U (" << realU << ") too big for compiled configuration ("
                      << kMaxMatrixElements / 2 << ")" << std::endl;
            return false;
        }
        if (realV > kMaxMatrixElements / 2) {
            std::cout << "Error: real variables for V (" << realV << ") too big for compiled configuration ("
                      << kMaxMatrixElements / 2 << ")" << std::endl;
            return false;
        }
        if (realU > kMaxRank / 2) {
            std::cout << "Error: real variables for W (" << realW << ") too big for compiled configuration ("
                      << kMaxRank / 2 << ")" << std::endl;
            return false;
        }
        const int limits[3] = {kMaxMatrixElements * (kMaxMatrixElements - 1) / 2,
                               kMaxMatrixElements * (kMaxMatrixElements - 1) / 2, kMaxRank * (kMaxRank - 1) / 2};
        const char *names[3] = {"U", "V", "W"};
        for (int c = 0; c < 3; c++) {
            int sub = maxSubexpressions(c);
            if (sub > limits[c]) {
                std::cout << "Error: max subexpressions for " << names[c] << " (" << sub
                          << ") too big for compiled configuration (" << limits[c] << ")" << std::endl;
                return false;
            }
        }
        return true;
    }

    void reduce(int maxNoImprovements, int startAdditions) {  // scheme_additions_reducer.cu:92-117
        initialize();
        auto startTime = Clock::now();
        std::vector<double> times;
        int noImprovements = 0;
        for (int iteration = 1; noImprovements < maxNoImprovements; iteration++) {
            auto t1 = Clock::now();
            runIteration(iteration);
            bool improved = updateBest(startAdditions);
            auto t2 = Clock::now();
            times.push_back(std::chrono::duration_cast<std::chrono::milliseconds>(t2 - t1).count() / 1000.0);
            report(startTime, iteration, times);
            if (improved) {
                noImprovements = 0;
            } else {
                noImprovements++;
                std::cout << "No improvements for " << noImprovements << " iterations" << std::endl;
            }
        }
    }

private:
    int maxReal(int c) const {  // SchemeInteger::getMaxRealVariables
        int best = 0;
        if (c == 2) {
            for (int i = 0; i < scheme_.nn[2]; i++) {
                int k = 0;
                for (int t = 0; t < m_; t++) k += scheme_.coefficient(2, t, i) != 0;
                best = std::max(best, k);
            }
        } else {
            for (int t = 0; t < m_; t++) {
                int k = 0;
                for (int i = 0; i < scheme_.nn[c]; i++) k += scheme_.coefficient(c, t, i) != 0;
                best = std::max(best, k);
            }
        }
        return best;
    }

    int maxSubexpressions(int c) const {  // SchemeInteger::getMaxSubexpressions
        auto check = [](int a, int b, bool &pos, bool &neg) {
            if (!a || !b) return;
            if (a < 0) { a = -a; b = -b; }
            if (b == 1) pos = true;
            if (b == -1) neg = true;
        };
        int total = 0;
        if (c == 2) {
            for (int a = 0; a < m_; a++)
                for (int b = a + 1; b < m_; b++) {
                    bool pos = false, neg = false;
                    for (int i = 0; i < scheme_.nn[2] && (!pos || !neg); i++)
                        check(scheme_.coefficient(2, a, i), scheme_.coefficient(2, b, i), pos, neg);
                    total += int(pos) + int(neg);
                }
        } else {
            for (int i1 = 0; i1 < scheme_.nn[c]; i1++)
                for (int i2 = i1 + 1; i2 < scheme_.nn[c]; i2++) {
                    bool pos = false, neg = false;
                    for (int t = 0; t < m_ && (!pos || !neg); t++)
                        check(scheme_.coefficient(c, t, i1), scheme_.coefficient(c, t, i2), pos, neg);
                    total += int(pos) + int(neg);
                }
        }
        return total;
    }

    Expressions naive(int c) const { return naiveOf(coef0_.data(), m_, c); }

    // copySchemeToReducers (scheme_additions_reducer.cu:463-492) of a scheme given as
    // coefficient rows [3][m_][64] with rank `rank` (a flipped scheme may have dropped rank).
    Expressions naiveOf(const int8_t *coef, int rank, int c) const {
        Expressions x;
        const int nn = scheme_.nn[c];
        auto at = [&](int cc, int t, int i) { return (int)coef[((size_t)cc * m_ + t) * 64 + i]; };
        if (c < 2) {
            x.real = nn;
            for (int t = 0; t < rank; t++) {
                std::vector<int> e;
                for (int i = 0; i < nn; i++) {
                    int v = at(c, t, i);
                    if (v) e.push_back(v > 0 ? i + 1 : -(i + 1));
                }
                x.e.push_back(e);
            }
        } else {
            x.real = rank;
            for (int i = 0; i < nn; i++) {
                std::vector<int> e;
                for (int t = 0; t < rank; t++) {
                    int v = at(2, t, i);
                    if (v) e.push_back(v > 0 ? t + 1 : -(t + 1));
                }
                x.e.push_back(e);
            }
        }
        return x;
    }

    static int additionsOf(const Expressions &x) {
        int a = (int)x.vars.size();
        for (auto &e : x.e) a += (int)e.size() - 1;
        return a;
    }

    void initialize() {  // scheme_additions_reducer.cu:234-258
        coef0_.assign((size_t)3 * m_ * 64, 0);
        for (int c = 0; c < 3; c++)
            for (int t = 0; t < m_; t++)
                for (int i = 0; i < scheme_.nn[c]; i++)
                    coef0_[((size_t)c * m_ + t) * 64 + i] = (int8_t)scheme_.coefficient(c, t, i);
        std::vector<int8_t> coef((size_t)schemesCount_ * 3 * m_ * 64, 0);
        for (int s = 0; s < schemesCount_; s++) std::copy(coef0_.begin(), coef0_.end(), coef.begin() + (size_t)s * coef0_.size());
        schemeCoef_ = coef;
        schemeRanks_.assign(schemesCount_, m_);
        bestCoef_ = coef0_;
        bestRank_ = m_;
        // One scheme and few reducers leave most SMs idle: wide blocks (results unchanged).
        fg_reducer_config cfg{count_, schemesCount_, (uint64_t)(long long)seed_, 0, 512};
        check(fg_reducer_create(&cfg, n1_, n2_, n3_, m_, coef.data(), &h_), "fg_reducer_create");
        for (int c = 0; c < 3; c++) {
            best_[c] = ReducerView();
            Expressions x = naive(c);
            best_[c].naive = additionsOf(x);
            best_[c].additions = best_[c].naive;
            best_[c].vars.assign(1000, 0);
            bestAdditions_[c] = best_[c].additions;
        }
        bestFresh_[0] = n1_ * n2_ * (n1_ * n2_ - 1);
        bestFresh_[1] = n2_ * n3_ * (n2_ * n3_ - 1);
        bestFresh_[2] = m_ * (m_ - 1);
        reducedAdditions_ = bestAdditions_[0] + bestAdditions_[1] + bestAdditions_[2];
        reducedFresh_ = bestFresh_[0] + bestFresh_[1] + bestFresh_[2];
        int realMax[3];
        for (int c = 0; c < 3; c++) {
            realMax[c] = 0;
            for (auto &e : naive(c).e) realMax[c] = std::max(realMax[c], (int)e.size());
        }
        std::cout << "Readed scheme params:" << std::endl;
        std::cout << "- dimensions: " << n1_ << "x" << n2_ << "x" << n3_ << std::endl;
        std::cout << "- multiplications (rank): " << m_ << std::endl;
        std::cout << "- naive additions (U / V / W / total): " << bestAdditions_[0] << " / " << bestAdditions_[1]
                  << " / " << bestAdditions_[2] << " / " << reducedAdditions_ << std::endl;
        std::cout << "- max real variables (U / V / W): " << realMax[0] << " / " << realMax[1] << " / " << realMax[2]
                  << std::endl;
        std::cout << "- max unique subexpressions (U / V / W): " << maxSubexpressions(0) << " / "
                  << maxSubexpressions(1) << " / " << maxSubexpressions(2) << std::endl;
        std::cout << std::endl;
    }

    void runIteration(int iteration) {  // reduceIteration, scheme_additions_reducer.cu:172-182
        if (maxFlips_ > 0 && iteration > 1)
            check(fg_reducer_flip(h_, maxFlips_, schemeRanks_.data(), schemeCoef_.data()), "fg_reducer_flip");
        int32_t fresh[3];
        std::vector<int32_t> vars(3 * 1000, 0);
        for (int c = 0; c < 3; c++) {
            fresh[c] = best_[c].fresh;
            std::copy(best_[c].vars.begin(), best_[c].vars.begin() + 2 * fresh[c], vars.begin() + c * 1000);
        }
        counts_.assign((size_t)count_ * 13, 0);
        scales_.assign((size_t)count_ * 3, 0);
        vars_.assign((size_t)count_ * 3 * 1000, 0);
        check(fg_reducer_run(h_, maxFlips_ == 0 ? 1 : 0, fresh, vars.data(), counts_.data(), scales_.data(), vars_.data()),
              "fg_reducer_run");
    }

    ReducerView view(int r, int c) const {
        ReducerView v;
        const int32_t *k = &counts_[(size_t)r * 13 + c * 4];
        v.additions = k[0];
        v.fresh = k[1];
        v.naive = k[2];
        v.mode = k[3];
        v.scale = scales_[(size_t)r * 3 + c];
        v.vars.assign(vars_.begin() + ((size_t)r * 3 + c) * 1000, vars_.begin() + ((size_t)r * 3 + c + 1) * 1000);
        return v;
    }

    bool updateBestIndependent() {  // scheme_additions_reducer.cu:272-339
        bool updated = false;
        for (int c = 0; c < 3; c++) {
            std::partial_sort(indices_[c].begin(), indices_[c].begin() + topCount_, indices_[c].end(), [&](int a, int b) {
                int aa = counts_[(size_t)a * 13 + c * 4], ab = counts_[(size_t)b * 13 + c * 4];
                if (aa != ab) return aa < ab;
                return counts_[(size_t)a * 13 + c * 4 + 1] < counts_[(size_t)b * 13 + c * 4 + 1];
            });
        }
        for (int c = 0; c < 3; c++) {
            ReducerView v = view(indices_[c][0], c);
            if (v.additions < bestAdditions_[c] || (v.additions == bestAdditions_[c] && v.fresh < bestFresh_[c])) {
                bestAdditions_[c] = v.additions;
                bestFresh_[c] = v.fresh;
                best_[c] = v;
                updated = true;
            }
        }
        return updated;
    }

    int total(int r, int field) const {  // U + V + W of one counts field (0 additions, 1 fresh)
        return counts_[(size_t)r * 13 + field] + counts_[(size_t)r * 13 + 4 + field] + counts_[(size_t)r * 13 + 8 + field];
    }

    bool updateBestTogether() {  // scheme_additions_reducer.cu:296-339: one reducer's U, V and W
        std::partial_sort(indices_[0].begin(), indices_[0].begin() + topCount_, indices_[0].end(), [&](int a, int b) {
            if (total(a, 0) != total(b, 0)) return total(a, 0) < total(b, 0);
            return total(a, 1) < total(b, 1);
        });
        const int top = indices_[0][0];
        const int additions = total(top, 0), freshVars = total(top, 1);
        if (additions < reducedAdditions_ || (additions == reducedAdditions_ && freshVars < reducedFresh_)) {
            for (int c = 0; c < 3; c++) {
                best_[c] = view(top, c);
                bestAdditions_[c] = best_[c].additions;
                bestFresh_[c] = best_[c].fresh;
            }
            const int s = top % schemesCount_;  // the scheme this reducer reduced
            bestCoef_.assign(schemeCoef_.begin() + (size_t)s * 3 * m_ * 64, schemeCoef_.begin() + (size_t)(s + 1) * 3 * m_ * 64);
            bestRank_ = schemeRanks_[s];
            return true;
        }
        return false;
    }

    bool updateBest(int startAdditions) {  // scheme_additions_reducer.cu:384-404
        bool updated = maxFlips_ == 0 ? updateBestIndependent() : updateBestTogether();
        int additions = bestAdditions_[0] + bestAdditions_[1] + bestAdditions_[2];
        int freshVars = bestFresh_[0] + bestFresh_[1] + bestFresh_[2];
        if (!updated) return false;
        if (additions < reducedAdditions_)
            std::cout << "Reduced scheme improved from " << reducedAdditions_ << " to " << additions
                      << " additions (fresh vars: " << freshVars << ")" << std::endl;
        else
            std::cout << "Reduced scheme improved from " << reducedFresh_ << " fresh vars to " << freshVars
                      << " fresh vars (additions: " << reducedAdditions_ << ")" << std::endl;
        reducedAdditions_ = additions;
        reducedFresh_ = freshVars;
        if (reducedAdditions_ < startAdditions || startAdditions == 0) save();
        return true;
    }

    void report(Clock::time_point startTime, int iteration, const std::vector<double> &times) {  // :406-476
        double elapsed = std::chrono::duration_cast<std::chrono::milliseconds>(Clock::now() - startTime).count() / 1000.0;
        double lastTime = times.back();
        double minTime = *std::min_element(times.begin(), times.end());
        double maxTime = *std::max_element(times.begin(), times.end());
        double meanTime = std::accumulate(times.begin(), times.end(), 0.0) / times.size();
        std::ostringstream dims;
        dims << n1_ << "x" << n2_ << "x" << n3_;
        std::cout << std::endl << std::left;
        std::cout << "+----------------------------------------------------------------------------------------------------------------------------+" << std::endl;
        std::cout << "| Size: " << std::setw(24) << dims.str() << "   Reducers: " << std::setw(20) << count_ << "   "
                  << "                                 Iteration: " << std::setw(12) << iteration << " |" << std::endl;
        std::cout << "| Rank: " << std::setw(24) << m_ << "   Schemes: " << std::setw(21) << schemesCount_ << "   "
                  << "                                 Elapsed: " << std::setw(14) << prettyTime(elapsed) << " |" << std::endl;
        std::cout << std::right;
        std::cout << "+================================+================================+================================+=========================+" << std::endl;
        std::cout << "|           Reducers U           |           Reducers V           |           Reducers W           |          Total          |" << std::endl;
        std::cout << "+------+-------+---------+-------+------+-------+---------+-------+------+-------+---------+-------+-------+---------+-------|" << std::endl;
        std::cout << "| mode | naive | reduced | fresh | mode | naive | reduced | fresh | mode | naive | reduced | fresh | naive | reduced | fresh |" << std::endl;
        std::cout << "+------+-------+---------+-------+------+-------+---------+-------+------+-------+---------+-------+-------+---------+-------+" << std::endl;
        for (int i = 0; i < topCount_ && i < count_; i++) {
            // --max-flips: the rows are whole reducers (scheme_additions_reducer.cu:353-354)
            const int k = maxFlips_ > 0 ? 0 : 1, l = maxFlips_ > 0 ? 0 : 2;
            ReducerView v[3] = {view(indices_[0][i], 0), view(indices_[k][i], 1), view(indices_[l][i], 2)};
            std::cout << "| ";
            for (int c = 0; c < 3; c++)
                std::cout << std::setw(4) << modeName(v[c].mode, v[c].scale) << "   " << std::setw(5) << v[c].naive
                          << "   " << std::setw(7) << v[c].additions << "   " << std::setw(5) << v[c].fresh << " | ";
            std::cout << std::setw(5) << v[0].naive + v[1].naive + v[2].naive << "   " << std::setw(7)
                      << v[0].additions + v[1].additions + v[2].additions << "   " << std::setw(5)
                      << v[0].fresh + v[1].fresh + v[2].fresh << " | " << std::endl;
        }
        std::cout << "+--------------------------------+--------------------------------+--------------------------------+-------------------------+" << std::endl;
        std::cout << "- iteration time (last / min / max / mean): " << prettyTime(lastTime) << " / " << prettyTime(minTime)
                  << " / " << prettyTime(maxTime) << " / " << prettyTime(meanTime) << std::endl;
        std::cout << "- best additions (U / V / W / total): " << bestAdditions_[0] << " / " << bestAdditions_[1] << " / "
                  << bestAdditions_[2] << " / " << reducedAdditions_ << std::endl;
        std::cout << "- best fresh vars (U / V / W / total): " << bestFresh_[0] << " / " << bestFresh_[1] << " / "
                  << bestFresh_[2] << " / " << reducedFresh_ << std::endl;
        std::cout << std::endl;
    }

    void save() const {  // scheme_additions_reducer.cu:478-513
        int naiveTotal = best_[0].naive + best_[1].naive + best_[2].naive;
        std::ostringstream p;
        p << out_ << "/" << n1_ << "x" << n2_ << "x" << n3_ << "_m" << m_ << "_cr" << reducedAdditions_ << "_fv"
          << reducedFresh_ << "_cn" << naiveTotal << "_ZT_reduced.json";
        std::ofstream f(p.str());
        f << "{" << std::endl;
        f << "    \"n\": [" << n1_ << ", " << n2_ << ", " << n3_ << "]," << std::endl;
        f << "    \"m\": " << m_ << "," << std::endl;
        f << "    \"z2\": false," << std::endl;
        f << "    \"complexity\": {\"naive\": " << naiveTotal << ", \"reduced\": " << reducedAdditions_ << "}," << std::endl;
        const char *names[3] = {"u", "v", "w"};
        for (int c = 0; c < 3; c++) {  // the best reducer's own scheme ("m" stays the input's, as the reference writes)
            Expressions x = naiveOf(bestCoef_.data(), bestRank_, c);
            for (int q = 0; q < best_[c].fresh; q++) x.replace(best_[c].vars[2 * q], best_[c].vars[2 * q + 1]);
            x.write(f, names[c], "    ");
            f << (c < 2 ? "," : "") << std::endl;
        }
        f << "}" << std::endl;
        f.close();
        std::cout << "Reduced scheme saved to \"" << p.str() << "\"" << std::endl;
    }

    int count_, schemesCount_, maxFlips_, seed_;
    std::string out_;
    bool z2input_;
    int topCount_ = 10;
    int n1_ = 0, n2_ = 0, n3_ = 0, m_ = 0;
    HostScheme scheme_;
    fg_reducer *h_ = nullptr;
    std::vector<int> indices_[3];
    ReducerView best_[3];
    int bestAdditions_[3] = {0, 0, 0}, bestFresh_[3] = {0, 0, 0};
    int reducedAdditions_ = 0, reducedFresh_ = 0;
    std::vector<int32_t> counts_, vars_;
    std::vector<float> scales_;
    std::vector<int8_t> coef0_, schemeCoef_, bestCoef_;  // input, every scheme of this iteration, the best's
    std::vector<int32_t> schemeRanks_;
    int bestRank_ = 0;
};

}  // namespace

int main(int argc, char *argv[]) {
    ArgParser parser("addition_reducer", "Find best additions number of the fast matrix multiplication scheme in parallel using CUDA");
    parser.add("-i", ArgType::String, "PATH", "path to init scheme(s)", "");
    parser.add("-o", ArgType::String, "PATH", "path to save schemes", "schemes/additions_reduced");
    parser.add("--count", ArgType::Natural, "INT", "number of parallel reducers", "32");
    parser.add("--schemes-count", ArgType::Natural, "INT", "number of parallel schemes", "1");
    parser.add("--block-size", ArgType::Natural, "INT", "number of cuda threads (accepted; the library sizes its launches)", "32");
    parser.add("--start-additions", ArgType::Natural, "INT", "upper bound of additions for check optimality", "0");
    parser.add("--max-flips", ArgType::Natural, "INT", "number of scheme flips", "0");
    parser.add("--max-no-improvements", ArgType::Natural, "INT", "max iterations without improvements", "3");
    parser.add("--seed", ArgType::Natural, "INT", "random seed", "0");
    parser.add("--z2-input", ArgType::Natural, "0|1", "accept schemes valid only modulo 2", "0");
    if (!parser.parse(argc, argv)) return 0;

    std::string inputPath = parser.get("-i");
    std::string outputPath = parser.get("-o");
    int count = std::stoi(parser.get("--count"));
    int schemesCount = std::stoi(parser.get("--schemes-count"));
    std::string blockSize = parser.get("--block-size");
    int maxNoImprovements = std::stoi(parser.get("--max-no-improvements"));
    int startAdditions = std::stoi(parser.get("--start-additions"));
    int maxFlips = std::stoi(parser.get("--max-flips"));
    int seed = std::stoi(parser.get("--seed"));
    bool z2input = parser.get("--z2-input") == "1";
    if (seed == 0) seed = (int)time(0);

    std::stringstream f;  // the reference's text layout, or JSON saved by a run
    std::string inputError;
    if (!openSchemeInput(inputPath, TextLayout::Reducer, f, inputError)) {
        std::cout << inputError << std::endl;
        return -1;
    }
    std::cout << "Compiled configuration:" << std::endl;
    std::cout << "- max expressions count (U / V / W): " << kMaxRank << " / " << kMaxRank << " / " << kMaxMatrixElements << std::endl;
    std::cout << "- max real variables (U / V / W): " << kMaxMatrixElements / 2 << " / " << kMaxMatrixElements / 2 << " / "
              << kMaxRank / 2 << std::endl;
    std::cout << "- max subexpressions (U / V / W): " << kMaxMatrixElements * (kMaxMatrixElements - 1) / 2 << " / "
              << kMaxMatrixElements * (kMaxMatrixElements - 1) / 2 << " / " << kMaxRank * (kMaxRank - 1) / 2 << std::endl;
    std::cout << "- max fresh variables (U / V / W): 250 / 250 / 500" << std::endl;
    std::cout << std::endl;
    std::cout << "Start additions reduction algorithm" << std::endl;
    std::cout << "- count: " << count << std::endl;
    std::cout << "- schemes count: " << schemesCount << std::endl;
    std::cout << "- output path: " << outputPath << std::endl;
    std::cout << "- block size: " << blockSize << std::endl;
    if (startAdditions > 0) std::cout << "- start additions: " << startAdditions << std::endl;
    if (maxFlips > 0) std::cout << "- max flips: " << maxFlips << std::endl;
    std::cout << "- max no improvements: " << maxNoImprovements << std::endl;
    std::cout << "- seed: " << seed << std::endl;
    std::cout << std::endl;

    if (maxFlips > 0 && schemesCount > count) {  // flipSchemesKernel reads states[s] of the reducers
        std::cout << "Error: --schemes-count must not exceed --count when --max-flips > 0" << std::endl;
        return -1;
    }
    SchemeAdditionsReducer reducer(count, schemesCount, maxFlips, seed, outputPath, z2input);
    bool correct = reducer.read(f);
    if (!correct) return -1;
    reducer.reduce(maxNoImprovements, startAdditions);
    return 0;
}
