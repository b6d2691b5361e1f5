#include "common.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>

namespace fgcli {

// ---------------------------------------------------------------- arguments
ArgParser::ArgParser(std::string name, std::string description)
    : name_(std::move(name)), description_(std::move(description)) {}

void ArgParser::add(const std::string &name, ArgType type, const std::string &meta, const std::string &description,
                    const std::string &value) {
    args_.push_back({name, meta, description, value, type});
}

static bool isNatural(const std::string &v) {
    for (char ch : v)
        if (ch < '0' || ch > '9') return false;
    return true;
}

static bool isReal(const std::string &v) {
    if (v.empty()) return false;
    bool point = false;
    for (size_t i = v[0] == '-' ? 1 : 0; i < v.size(); i++) {
        if (v[i] == '.') {
            if (point) return false;
            point = true;
        } else if (v[i] < '0' || v[i] > '9') {
            return false;
        }
    }
    return true;
}

bool ArgParser::parse(int argc, char **argv) {
    if (argc == 2 && std::string(argv[1]) == "--help") {
        help();
        return false;
    }
    if (argc % 2 != 1) {
        std::cerr << "Invalid number of arguments" << std::endl;
        help();
        return false;
    }
    std::unordered_map<std::string, const Arg *> byName;
    for (const Arg &a : args_) {
        byName[a.name] = &a;
        if (!a.value.empty()) parsed_[a.name] = a.value;
    }
    for (int i = 1; i < argc; i += 2) {
        std::string name = argv[i];
        auto it = byName.find(name);
        if (it == byName.end()) {
            std::cerr << "unknown argument \"" << name << "\"" << std::endl;
            return false;
        }
        std::string value = argv[i + 1];
        parsed_[name] = value;
        const Arg &a = *it->second;
        if (a.type == ArgType::Natural && !isNatural(value)) {
            std::cerr << "value for arg \"" << name << "\" is not natural (" << value << ")" << std::endl;
            return false;
        }
        if (a.type == ArgType::Real && !isReal(value)) {
            std::cerr << "value for arg \"" << name << "\" is not real (" << value << ")" << std::endl;
            return false;
        }
    }
    for (const Arg &a : args_)
        if (a.value.empty() && !parsed_.count(a.name)) {
            std::cerr << "no value for argument \"" << a.name << "\"" << std::endl;
            return false;
        }
    return true;
}

std::string ArgParser::get(const std::string &name) const {
    auto it = parsed_.find(name);
    if (it == parsed_.end()) throw std::runtime_error("no parsed value for argument \"" + name + "\"");
    return it->second;
}

void ArgParser::help() const {
    std::cout << description_ << std::endl << "Usage: ./" << name_;
    for (const Arg &a : args_) {
        if (!a.value.empty()) std::cout << " [" << a.name << " " << a.value << "]";
        else std::cout << " " << a.name << " " << a.meta;
    }
    std::cout << std::endl << std::endl << "Arguments description:" << std::endl;
    for (const Arg &a : args_) {
        std::cout << a.name << ": " << a.description;
        if (!a.value.empty()) std::cout << " (default: " << a.value << ")";
        std::cout << std::endl;
    }
}

// ---------------------------------------------------------------- formatting
std::string key(int n1, int n2, int n3, bool sorted, bool withZeros) {
    int n[3] = {n1, n2, n3};
    if (sorted) std::sort(n, n + 3);
    std::ostringstream ss;
    for (int i = 0; i < 3; i++) {
        if (withZeros) ss << std::setfill('0') << std::setw(2);
        ss << n[i];
        if (i < 2) ss << "x";
    }
    return ss.str();
}

std::string prettyTime(double elapsed) {
    std::ostringstream ss;
    if (elapsed < 60) {
        ss << std::setprecision(3) << std::fixed << elapsed;
    } else {
        int seconds = int(elapsed + 0.5);
        ss << std::setw(2) << std::setfill('0') << seconds / 3600 << ":";
        ss << std::setw(2) << std::setfill('0') << (seconds % 3600) / 60 << ":";
        ss << std::setw(2) << std::setfill('0') << seconds % 60;
    }
    return ss.str();
}

std::string prettyInt(int value) {
    std::ostringstream ss;
    if (value < 1000) ss << value;
    else if (value < 1000000) ss << std::setprecision(2) << std::fixed << value / 1000.0 << "K";
    else ss << std::setprecision(2) << std::fixed << value / 1000000.0 << "M";
    return ss.str();
}

// Best known ranks (sorted shape key -> rank) as the walk report prints them;
// a common table plus ring-specific entries.
static const char *kKnownCommon =
    "2x2x2:7 2x2x3:11 2x2x4:14 2x2x5:18 2x2x6:21 2x2x7:25 2x2x8:28 2x2x9:32 2x2x10:35 2x2x11:39 2x2x12:42 "
    "2x2x13:46 2x2x14:49 2x2x15:53 2x2x16:56 2x3x3:15 2x3x4:20 2x3x5:25 2x3x6:30 2x3x7:35 2x3x8:40 2x3x9:45 "
    "2x3x10:50 2x3x11:55 2x3x12:60 2x3x13:65 2x3x14:70 2x3x15:75 2x3x16:80 2x4x4:26 2x4x5:32 2x4x6:39 2x4x7:45 "
    "2x4x8:51 2x4x9:59 2x4x10:64 2x4x11:71 2x4x12:77 2x4x13:83 2x4x14:90 2x4x15:96 2x4x16:102 2x5x5:40 2x5x6:47 "
    "2x5x7:55 2x5x8:63 2x5x9:72 2x5x10:79 2x5x11:87 2x5x12:94 2x6x6:56 2x6x7:66 2x6x8:75 2x6x9:86 2x6x10:94 "
    "2x7x7:76 2x7x8:88 2x7x9:99 2x8x8:100 3x3x3:23 3x3x4:29 3x3x5:36 3x3x6:40 3x3x7:49 3x3x8:55 3x3x9:63 "
    "3x3x10:69 3x3x11:76 3x3x12:80 3x3x13:89 3x3x14:95 3x3x15:103 3x3x16:109 3x4x4:38 3x4x5:47 3x4x6:54 3x4x7:63 "
    "3x4x8:73 3x4x9:83 3x4x10:92 3x4x11:101 3x4x12:108 3x4x13:117 3x4x14:126 3x4x15:136 3x4x16:146 3x5x5:58 "
    "3x5x6:68 3x5x7:79 3x5x8:90 3x5x9:104 3x5x10:115 3x5x11:126 3x5x12:136 3x6x6:80 3x6x7:94 3x6x8:108 3x6x9:120 "
    "3x6x10:134 3x7x7:111 3x7x8:126 3x7x9:142 3x8x8:145 4x4x4:48 4x4x5:61 4x4x6:73 4x4x7:85 4x4x8:96 4x4x9:104 "
    "4x4x10:120 4x4x11:130 4x4x12:142 4x4x13:152 4x4x14:165 4x4x15:177 4x4x16:189 4x5x5:76 4x5x6:90 4x5x7:104 "
    "4x5x8:118 4x5x9:136 4x5x10:151 4x5x11:165 4x5x12:179 4x6x6:105 4x6x7:123 4x6x8:140 4x6x9:159 4x6x10:175 "
    "4x7x7:144 4x7x8:164 4x7x9:186 4x8x8:182 5x5x5:93 5x5x6:110 5x5x7:127 5x5x8:144 5x5x9:167 5x5x10:184 "
    "5x5x11:202 5x5x12:220 5x6x6:130 5x6x7:150 5x6x8:170 5x6x9:197 5x6x10:217 5x7x7:176 5x7x8:205 5x7x9:229 "
    "5x8x8:230 6x6x6:153 6x6x7:183 6x6x8:203 6x6x9:225 6x6x10:247 6x7x7:215 6x7x8:239 6x7x9:268 6x8x8:266 "
    "7x7x7:249 7x7x8:277 7x7x9:315 7x8x8:306 8x8x8:336";
static const char *kKnownZT =
    "2x4x5:33 2x4x10:65 2x4x13:84 2x5x7:57 2x5x8:65 2x5x10:80 2x6x6:57 2x6x7:68 2x6x8:77 2x7x7:77 2x7x8:90 "
    "2x7x9:102 3x3x6:43 3x3x7:51 3x3x8:58 3x3x9:65 3x3x10:72 3x3x11:79 3x3x12:86 3x3x13:94 3x3x14:101 3x3x15:108 "
    "3x3x16:115 3x4x6:56 3x4x7:64 3x4x8:74 3x4x9:84 3x4x10:93 3x4x11:102 3x4x12:111 3x4x13:120 3x4x14:128 "
    "3x4x15:138 3x4x16:148 3x5x6:70 3x5x7:83 3x5x8:94 3x5x9:105 3x5x10:116 3x5x11:128 3x5x12:140 3x6x6:85 "
    "3x6x7:99 3x6x8:112 3x6x9:126 3x6x10:140 3x7x7:115 3x7x8:128 3x7x9:147 3x8x8:148 4x4x4:49 4x4x9:110 "
    "4x4x10:122 4x4x11:134 4x4x12:145 4x4x13:157 4x4x14:169 4x4x15:181 4x4x16:192 4x5x9:137 4x6x9:160 4x7x7:145 "
    "4x7x9:187 5x7x8:206 5x7x9:231 6x6x10:252 7x7x7:250 7x7x8:279 7x7x9:316 7x8x8:310 8x8x8:343";
static const char *kKnownZ2 =
    "2x4x5:33 2x4x10:65 2x4x13:84 2x5x10:80 2x7x9:101 3x3x6:42 3x3x8:56 3x3x9:64 3x3x10:71 3x3x11:78 3x3x12:84 "
    "3x3x13:91 3x3x14:98 3x3x15:105 3x3x16:112 3x4x7:64 3x4x13:118 3x4x14:128 3x4x15:137 3x6x6:84 3x6x7:96 "
    "3x6x9:122 3x6x10:136 3x7x8:128 3x7x9:143 4x4x4:47 4x4x5:60 4x4x8:94 4x4x9:107 4x4x11:132 4x4x12:141 "
    "4x4x13:154 4x4x14:167 4x4x15:179 4x4x16:188 4x5x5:73 4x5x6:89 4x5x9:133 4x5x10:146 4x5x11:162 4x5x12:177 "
    "4x7x9:187 5x5x9:166 5x5x10:183 5x5x11:200 5x5x12:217 6x6x10:252 7x7x7:248 7x7x8:275 7x7x9:313 7x8x8:302 "
    "8x8x8:329";

static void parseKnown(const char *text, std::unordered_map<std::string, int> &out) {
    std::istringstream ss(text);
    std::string tok;
    while (ss >> tok) {
        size_t c = tok.find(':');
        out[tok.substr(0, c)] = std::atoi(tok.c_str() + c + 1);
    }
}

const std::unordered_map<std::string, int> &knownRanks(bool zt) {
    static std::unordered_map<std::string, int> z2, t;
    if (z2.empty()) {
        parseKnown(kKnownCommon, z2);
        parseKnown(kKnownCommon, t);
        parseKnown(kKnownZ2, z2);
        parseKnown(kKnownZT, t);
    }
    return zt ? t : z2;
}

// ---------------------------------------------------------------- schemes
void HostScheme::resize() {
    for (int c = 0; c < 3; c++) {
        v[c].assign(kMaxRank, 0);
        s[c].assign(kMaxRank, 0);
        ok[c].assign(kMaxRank, 1);
        t2[c].assign(kMaxRank, 0);
    }
}

bool HostScheme::read(std::istream &is, bool checkValidity) {
    int a = 0, b = 0, c = 0, mm = 0;
    is >> a >> b >> c >> mm;
    return readBody(is, a, b, c, mm, checkValidity);
}

bool HostScheme::readBody(std::istream &is, int n1, int n2, int n3, int mm, bool checkValidity) {
    if (n1 * n2 > kMaxMatrixElements || n2 * n3 > kMaxMatrixElements || n3 * n1 > kMaxMatrixElements || mm > kMaxRank) {
        printf("%s::read(is): invalid scheme sizes (%d, %d, %d, %d)\n", zt ? "SchemeInteger" : "SchemeZ2", n1, n2, n3, mm);
        return false;
    }
    resize();
    n[0] = n1; n[1] = n2; n[2] = n3;
    m = mm;
    for (int i = 0; i < 3; i++) {
        nn[i] = n[i] * n[(i + 1) % 3];
        for (int t = 0; t < m; t++) {
            v[i][t] = s[i][t] = 0;
            ok[i][t] = 1;
            for (int j = 0; j < nn[i]; j++) {
                int value = 0;
                is >> value;
                const uint64_t bit = (uint64_t)1 << j;
                if (!zt) {
                    if (std::abs(value) % 2) v[i][t] |= bit;
                } else if (value == 0) {
                    v[i][t] &= ~bit; s[i][t] &= ~bit;
                } else if (value == 1) {
                    v[i][t] |= bit; s[i][t] &= ~bit;
                } else if (value == -1) {
                    v[i][t] |= bit; s[i][t] |= bit;
                } else {
                    ok[i][t] = 0;  // Addition::set (addition.cu:41-60)
                    printf("invalid set (%d, %d)\n", j, value);
                }
            }
        }
    }
    if (zt) fixSigns();
    initFlips();
    return !checkValidity || validate();
}

void HostScheme::initFlips() {
    for (int c = 0; c < 3; c++) {
        lists[c].clear();
        for (int a = 0; a < m; a++)
            for (int b = a + 1; b < m; b++)
                if (v[c][a] == v[c][b] && s[c][a] == s[c][b] && lists[c].size() < FG_LIST_CAP)
                    lists[c].push_back(((uint32_t)a << 16) | (uint32_t)b);
    }
}

bool HostScheme::fixSigns() {  // scheme_integer.cu:398-425
    auto fp = [](uint64_t vv, uint64_t ss) { return vv == 0 || (vv & ~(vv & (vv - 1)) & ~ss); };
    bool changed = false;
    for (int t = 0; t < m; t++) {
        bool pi = fp(v[0][t], s[0][t]), pj = fp(v[1][t], s[1][t]);
        if (pi && pj) continue;
        int c0 = (!pi && !pj) ? 0 : (!pi ? 0 : 1), c1 = (!pi && !pj) ? 1 : 2;
        s[c0][t] = ~s[c0][t] & v[c0][t];
        s[c1][t] = ~s[c1][t] & v[c1][t];
        changed = true;
    }
    return changed;
}

void HostScheme::removeZeroes() {
    if (!zt) {  // scheme_z2.cu:152-164
        while (m > 0 && !nonzero(m - 1)) m--;
        for (int t = 0; t < m; t++)
            if (!nonzero(t)) {
                m--;
                for (int c = 0; c < 3; c++) { v[c][t] = v[c][m]; s[c][t] = s[c][m]; ok[c][t] = ok[c][m]; }
            }
        return;
    }
    for (int t = 0; t < m; t++) {  // scheme_integer.cu:240-251
        if (nonzero(t)) continue;
        m--;
        for (int c = 0; c < 3; c++) { v[c][t] = v[c][m]; s[c][t] = s[c][m]; ok[c][t] = ok[c][m]; }
        t--;
    }
}

void HostScheme::removeAt(int t) {
    m--;
    if (t == m) return;
    for (int c = 0; c < 3; c++) { v[c][t] = v[c][m]; s[c][t] = s[c][m]; ok[c][t] = ok[c][m]; }
}

void HostScheme::reduceZ2(int i, int a, int b) {  // scheme_z2.cu:631-641
    v[i][a] ^= v[i][b];
    bool zero = !v[i][a];
    removeAt(b);
    if (zero) removeZeroes();
    initFlips();
}

void HostScheme::reduceTern(int i, int a, int b, bool subtract) {  // scheme_integer.cu:549-571
    uint64_t va = v[i][a], sa = s[i][a], vb = v[i][b], sb = s[i][b];
    uint64_t sv1 = sa & va, sv2 = subtract ? (~sb & vb) : (sb & vb);
    ok[i][a] = subtract ? !(va & vb & (sa ^ sb)) : !(va & vb & ~(sa ^ sb));
    v[i][a] = va ^ vb;
    s[i][a] = (sv1 | sv2) & v[i][a];
    bool zero = !v[i][a];
    removeAt(b);
    if (zero) removeZeroes();
    initFlips();
}

bool HostScheme::tryReduce() {
    if (!zt) {  // scheme_z2.cu:1127-1154
        for (uint32_t p : lists[0]) {
            int a = p >> 16, b = p & 0xFFFF;
            if (v[1][a] == v[1][b]) { reduceZ2(2, a, b); return true; }
            if (v[2][a] == v[2][b]) { reduceZ2(1, a, b); return true; }
        }
        for (uint32_t p : lists[1]) {
            int a = p >> 16, b = p & 0xFFFF;
            if (v[2][a] == v[2][b]) { reduceZ2(0, a, b); return true; }
        }
        return false;
    }
    // scheme_integer.cu:1062-1101
    auto fp = [](uint64_t vv, uint64_t ss) { return vv == 0 || (vv & ~(vv & (vv - 1)) & ~ss); };
    auto limitSum = [&](int c, int a, int b, bool f) {
        if (v[c][a] & v[c][b] & ~(s[c][a] ^ s[c][b])) return false;
        if (!f) return true;
        uint64_t sv = v[c][a] ^ v[c][b];
        return fp(sv, ((s[c][a] & v[c][a]) | (s[c][b] & v[c][b])) & sv);
    };
    auto limitSub = [&](int c, int a, int b, bool f) {
        if (v[c][a] & v[c][b] & (s[c][a] ^ s[c][b])) return false;
        if (!f) return true;
        uint64_t sv = v[c][a] ^ v[c][b];
        return fp(sv, ((s[c][a] & v[c][a]) | (~s[c][b] & v[c][b])) & sv);
    };
    auto compare = [&](int c, int a, int b) {
        if (v[c][a] != v[c][b]) return 0;
        if (s[c][a] == s[c][b]) return 1;
        if (s[c][a] == (~s[c][b] & v[c][b])) return -1;
        return 0;
    };
    for (uint32_t p : lists[0]) {
        int a = p >> 16, b = p & 0xFFFF;
        if (v[1][a] == v[1][b] && s[1][a] == s[1][b] && limitSum(2, a, b, false)) { reduceTern(2, a, b, false); return true; }
        int cmp2 = compare(2, a, b);
        if (cmp2 == 1 && limitSum(1, a, b, true)) { reduceTern(1, a, b, false); return true; }
        if (cmp2 == -1 && limitSub(1, a, b, true)) { reduceTern(1, a, b, true); return true; }
    }
    for (uint32_t p : lists[1]) {
        int a = p >> 16, b = p & 0xFFFF;
        int cmp2 = compare(2, a, b);
        if (cmp2 == 1 && limitSum(0, a, b, true)) { reduceTern(0, a, b, false); return true; }
        if (cmp2 == -1 && limitSub(0, a, b, true)) { reduceTern(0, a, b, true); return true; }
    }
    return false;
}

int HostScheme::coefficient(int c, int t, int entry) const {
    int x = (int)((v[c][t] >> entry) & 1);
    if (zb && ((t2[c][t] >> entry) & 1)) x *= 2;
    return ((s[c][t] >> entry) & 1) ? -x : x;
}

bool HostScheme::validate() const {
    for (int i = 0; i < nn[0]; i++)
        for (int j = 0; j < nn[1]; j++)
            for (int k = 0; k < nn[2]; k++) {
                int target = (i % n[1] == j / n[2]) && (i / n[1] == k % n[0]) && (j % n[2] == k / n[0]);
                int e = 0;
                for (int t = 0; t < m; t++) {
                    int p = coefficient(0, t, i) * coefficient(1, t, j) * coefficient(2, t, k);
                    e = zt ? e + p : (e ^ (p & 1));
                }
                if (e != target) return false;
            }
    if (zt)
        for (int t = 0; t < m; t++)
            for (int c = 0; c < 3; c++)
                if (!ok[c][t]) return false;
    return true;
}

int HostScheme::complexity() const {
    int count = 0;
    for (int t = 0; t < m; t++)
        for (int c = 0; c < 3; c++) count += __builtin_popcountll(v[c][t]);
    return count - 2 * m - nn[2];
}

// Scheme JSON exactly as SchemeZ2::save / SchemeInteger::save write it
// (scheme_z2.cu:1327-1364, scheme_integer.cu:1247-1274).
void HostScheme::saveJson(const std::string &path) const {
    std::ofstream f(path);
    f << "{" << std::endl;
    f << "    \"n\": [" << n[0] << ", " << n[1] << ", " << n[2] << "]," << std::endl;
    f << "    \"m\": " << m << "," << std::endl;
    f << "    \"z2\": " << (zt || zb ? "false" : "true") << "," << std::endl;
    f << "    \"complexity\": " << complexity() << "," << std::endl;
    const char *names[3] = {"u", "v", "w"};
    for (int c = 0; c < 3; c++) {
        f << "    \"" << names[c] << "\": [" << std::endl;
        for (int t = 0; t < m; t++) {
            f << "        [";
            for (int e = 0; e < nn[c]; e++) {
                if (e > 0) f << ", ";
                f << (zt || zb ? coefficient(c, t, e) : (int)((v[c][t] >> e) & 1));
            }
            f << "]" << (t < m - 1 ? "," : "") << std::endl;
        }
        f << "    ]";
        if (c < 2) f << "," << std::endl;
    }
    f << std::endl << "}" << std::endl;
}

void toRecords(const HostScheme &src, fg_records &rec, int w, int cap, bool withLists) {
    for (int c = 0; c < 3; c++) rec.n[w * 3 + c] = src.n[c];
    rec.m[w] = src.m;
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < cap; t++) {
            size_t q = ((size_t)w * 3 + c) * cap + t;
            bool in = t < src.m;
            rec.fac[q] = in ? src.v[c][t] : 0;
            if (rec.sgn) rec.sgn[q] = in ? src.s[c][t] : 0;
            if (rec.valid) rec.valid[q] = in ? src.ok[c][t] : 0;
        }
    for (int c = 0; c < 3; c++) {
        int L = withLists ? (int)src.lists[c].size() : 0;
        rec.list_size[w * 3 + c] = L;
        uint32_t *dst = rec.list_pairs + ((size_t)w * 3 + c) * FG_LIST_CAP;
        for (int q = 0; q < FG_LIST_CAP; q++) dst[q] = q < L ? src.lists[c][q] : 0;
    }
}

HostScheme fromRecords(const fg_records &rec, int w, int cap, bool zt, bool best) {
    HostScheme h;
    h.zt = zt;
    h.resize();
    for (int c = 0; c < 3; c++) h.n[c] = rec.n[w * 3 + c];
    for (int c = 0; c < 3; c++) h.nn[c] = h.n[c] * h.n[(c + 1) % 3];
    h.m = best ? rec.best_m[w] : rec.m[w];
    const uint64_t *fv = best ? rec.best_fac : rec.fac;
    const uint64_t *fs = best ? rec.best_sgn : rec.sgn;
    const uint8_t *fk = best ? rec.best_valid : rec.valid;
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < h.m; t++) {
            size_t q = ((size_t)w * 3 + c) * cap + t;
            h.v[c][t] = fv[q];
            h.s[c][t] = zt && fs ? fs[q] : 0;
            h.ok[c][t] = zt && fk ? fk[q] : 1;
        }
    return h;
}

HostScheme fetchScheme(fg_handle *hd, int w, int cap, bool zt, bool best) {
    HostScheme h;
    h.zt = zt;
    h.resize();
    std::vector<uint64_t> fv(3 * (size_t)cap), fs(3 * (size_t)cap);
    std::vector<uint8_t> fk(3 * (size_t)cap);
    int m = 0;
    check(fg_get_scheme(hd, w, best, h.n, &m, fv.data(), zt ? fs.data() : nullptr, zt ? fk.data() : nullptr),
          "fg_get_scheme");
    for (int c = 0; c < 3; c++) h.nn[c] = h.n[c] * h.n[(c + 1) % 3];
    h.m = m;
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < m; t++) {
            h.v[c][t] = fv[(size_t)c * cap + t];
            h.s[c][t] = zt ? fs[(size_t)c * cap + t] : 0;
            h.ok[c][t] = zt ? fk[(size_t)c * cap + t] : 1;
        }
    return h;
}

HostScheme fetchSchemeZB(fg_handle *hd, int w, int cap, bool best) {
    HostScheme h;
    h.zt = false;
    h.zb = true;
    h.resize();
    std::vector<uint64_t> fv(3 * (size_t)cap), fs(3 * (size_t)cap), f2(3 * (size_t)cap);
    int m = 0;
    check(fg_get_scheme_zb(hd, w, best, h.n, &m, fv.data(), fs.data(), f2.data()), "fg_get_scheme_zb");
    for (int c = 0; c < 3; c++) h.nn[c] = h.n[c] * h.n[(c + 1) % 3];
    h.m = m;
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < m; t++) {
            h.v[c][t] = fv[(size_t)c * cap + t];
            h.s[c][t] = fs[(size_t)c * cap + t];
            h.t2[c][t] = f2[(size_t)c * cap + t];
        }
    return h;
}

std::string ringName(bool zt) { return zt ? "ZT" : "Z2"; }

bool check(fg_status st, const char *what) {
    if (st == FG_OK) return true;
    std::cerr << what << " failed: " << fg_last_error() << std::endl;
    std::exit(EXIT_FAILURE);
}

}  // namespace fgcli
