// Host-side pieces shared by the three executables (flip_graph,
// complexity_minimizer, additions_reducer): the reference's flag grammar,
// scheme text input, JSON output and the small amount of scheme algebra the
// reference runs on the host (reading, tryReduce to a fixpoint, validation).
// Device work goes through the C ABI in include/flipgraph.h.
#pragma once
#include <cstdint>
#include <iosfwd>
#include <string>
#include <unordered_map>
#include <vector>

#include "flipgraph.h"

namespace fgcli {

constexpr int kMaxRank = FG_MAX_RANK;
constexpr int kMaxMatrixElements = 64;

// ---------------------------------------------------------------- arguments
// Flag/value pairs only (argc must be odd), `--help` alone, typed values:
// Natural = digits only, Real = optional leading '-', digits, at most one '.'
// (the reference's ArgParser, arg_parser.cu:16-57,108-135).
enum class ArgType { String, Natural, Real };

class ArgParser {
public:
    ArgParser(std::string name, std::string description);
    void add(const std::string &name, ArgType type, const std::string &meta, const std::string &description,
             const std::string &value = "");
    bool parse(int argc, char **argv);
    std::string get(const std::string &name) const;
    void help() const;

private:
    struct Arg {
        std::string name, meta, description, value;
        ArgType type;
    };
    std::string name_, description_;
    std::vector<Arg> args_;
    std::unordered_map<std::string, std::string> parsed_;
};

// ---------------------------------------------------------------- formatting
std::string key(int n1, int n2, int n3, bool sorted = true, bool withZeros = false);  // utils.cu:3-25
std::string prettyTime(double seconds);                                                // utils.cu:31-49
std::string prettyInt(int value);                                                      // utils.cu:51-61

// Best known ranks per sorted shape key, for the walk report's "known" column.
const std::unordered_map<std::string, int> &knownRanks(bool zt);

// ---------------------------------------------------------------- schemes
// A scheme on the host in the library's record layout: Z2 factors are
// bitmasks in v; ZT factors are (v, s, ok) as the reference's Addition.
struct HostScheme {
    bool zt = true;
    bool zb = false;  // integers with |c| <= 2: t2 marks the entries of magnitude 2 (v nonzero, s negative)
    int n[3] = {0, 0, 0}, nn[3] = {0, 0, 0}, m = 0;
    std::vector<uint64_t> v[3], s[3];
    std::vector<uint8_t> ok[3];
    std::vector<uint64_t> t2[3];
    std::vector<uint32_t> lists[3];

    // "n1 n2 n3 m" followed by the U, V, W rows (scheme_z2.cu:72-96, scheme_integer.cu:81-107).
    bool read(std::istream &is, bool checkValidity);
    bool readBody(std::istream &is, int n1, int n2, int n3, int m, bool checkValidity);
    void initFlips();
    bool tryReduce();
    bool validate() const;
    int complexity() const;
    int coefficient(int c, int t, int entry) const;
    void saveJson(const std::string &path) const;

    // Reference semantics helpers.
    void removeZeroes();
    void removeAt(int t);
    bool fixSigns();
    void resize();  // allocates kMaxRank slots per component

private:
    bool nonzero(int t) const { return v[0][t] && v[1][t] && v[2][t]; }
    void reduceZ2(int i, int a, int b);
    void reduceTern(int i, int a, int b, bool subtract);
};

// Copies scheme `src` into walk slot w of host records with `cap` slots.
void toRecords(const HostScheme &src, fg_records &rec, int w, int cap, bool withLists);
// Walk w's scheme (current, or best when best = true) from host records.
HostScheme fromRecords(const fg_records &rec, int w, int cap, bool zt, bool best);
// One walk's scheme straight from the library.
HostScheme fetchScheme(fg_handle *h, int w, int cap, bool zt, bool best);
// One ZB walk's scheme (integers with |c| <= 2).
HostScheme fetchSchemeZB(fg_handle *h, int w, int cap, bool best);

std::string ringName(bool zt);
bool check(fg_status st, const char *what);

}  // namespace fgcli
