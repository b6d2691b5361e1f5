#include "scheme_io.h"

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <dirent.h>
#include <fstream>
#include <sys/stat.h>

namespace fgcli {

namespace {

// ---------------------------------------------------------------- JSON
// A small JSON reader: objects, arrays, numbers, strings, true/false/null.
struct JValue {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    double number = 0;
    bool integral = false;
    long long integer = 0;
    std::string str;
    std::vector<JValue> items;
    std::vector<std::pair<std::string, JValue>> fields;

    const JValue *field(const std::string &key) const {
        for (const auto &f : fields)
            if (f.first == key) return &f.second;
        return nullptr;
    }
};

class JsonReader {
public:
    explicit JsonReader(const std::string &text) : t_(text) {}

    bool document(JValue &v, std::string &error) {
        if (!value(v, 0)) {
            error = err_;
            return false;
        }
        skip();
        if (p_ != t_.size()) {
            error = at("trailing characters after the JSON value");
            return false;
        }
        return true;
    }

private:
    const std::string &t_;
    size_t p_ = 0;
    std::string err_;

    std::string at(const std::string &what) const {
        size_t line = 1 + std::count(t_.begin(), t_.begin() + std::min(p_, t_.size()), '\n');
        return what + " (line " + std::to_string(line) + ")";
    }
    bool fail(const std::string &what) {
        if (err_.empty()) err_ = at(what);
        return false;
    }
    void skip() {
        while (p_ < t_.size() && std::isspace((unsigned char)t_[p_])) p_++;
    }
    bool literal(const char *word) {
        size_t n = std::char_traits<char>::length(word);
        if (t_.compare(p_, n, word) != 0) return false;
        p_ += n;
        return true;
    }

    bool value(JValue &v, int depth) {
        if (depth > 64) return fail("JSON nested too deeply");
        skip();
        if (p_ >= t_.size()) return fail("unexpected end of JSON");
        const char ch = t_[p_];
        if (ch == '{') return object(v, depth);
        if (ch == '[') return array(v, depth);
        if (ch == '"') {
            v.kind = JValue::String;
            return string(v.str);
        }
        if (literal("true")) { v.kind = JValue::Bool; v.number = 1; return true; }
        if (literal("false")) { v.kind = JValue::Bool; v.number = 0; return true; }
        if (literal("null")) { v.kind = JValue::Null; return true; }
        if (ch == '-' || std::isdigit((unsigned char)ch)) return number(v);
        return fail(std::string("unexpected character '") + ch + "' in JSON");
    }

    bool number(JValue &v) {
        const size_t start = p_;
        if (t_[p_] == '-') p_++;
        bool digits = false, frac = false;
        while (p_ < t_.size() && std::isdigit((unsigned char)t_[p_])) { p_++; digits = true; }
        if (p_ < t_.size() && t_[p_] == '.') {
            frac = true;
            p_++;
            while (p_ < t_.size() && std::isdigit((unsigned char)t_[p_])) p_++;
        }
        if (p_ < t_.size() && (t_[p_] == 'e' || t_[p_] == 'E')) {
            frac = true;
            p_++;
            if (p_ < t_.size() && (t_[p_] == '+' || t_[p_] == '-')) p_++;
            while (p_ < t_.size() && std::isdigit((unsigned char)t_[p_])) p_++;
        }
        if (!digits) return fail("malformed number in JSON");
        const std::string s = t_.substr(start, p_ - start);
        v.kind = JValue::Number;
        v.number = std::strtod(s.c_str(), nullptr);
        v.integral = !frac;
        if (v.integral) v.integer = std::strtoll(s.c_str(), nullptr, 10);
        return true;
    }

    bool string(std::string &out) {
        p_++;  // opening quote
        out.clear();
        while (p_ < t_.size() && t_[p_] != '"') {
            if (t_[p_] == '\\') {
                if (++p_ >= t_.size()) break;
                const char e = t_[p_];
                if (e == 'u') {  // keys here are ASCII; keep the escape verbatim
                    out += "\\u";
                } else {
                    out += e == 'n' ? '\n' : e == 't' ? '\t' : e == 'r' ? '\r' : e == 'b' ? '\b' : e == 'f' ? '\f' : e;
                }
                p_++;
                continue;
            }
            out += t_[p_++];
        }
        if (p_ >= t_.size()) return fail("unterminated string in JSON");
        p_++;
        return true;
    }

    bool array(JValue &v, int depth) {
        v.kind = JValue::Array;
        p_++;
        skip();
        if (p_ < t_.size() && t_[p_] == ']') { p_++; return true; }
        for (;;) {
            v.items.emplace_back();
            if (!value(v.items.back(), depth + 1)) return false;
            skip();
            if (p_ < t_.size() && t_[p_] == ',') { p_++; continue; }
            if (p_ < t_.size() && t_[p_] == ']') { p_++; return true; }
            return fail("expected ',' or ']' in JSON array");
        }
    }

    bool object(JValue &v, int depth) {
        v.kind = JValue::Object;
        p_++;
        skip();
        if (p_ < t_.size() && t_[p_] == '}') { p_++; return true; }
        for (;;) {
            skip();
            if (p_ >= t_.size() || t_[p_] != '"') return fail("expected a key in JSON object");
            std::string key;
            if (!string(key)) return false;
            skip();
            if (p_ >= t_.size() || t_[p_] != ':') return fail("expected ':' in JSON object");
            p_++;
            v.fields.emplace_back(key, JValue());
            if (!value(v.fields.back().second, depth + 1)) return false;
            skip();
            if (p_ < t_.size() && t_[p_] == ',') { p_++; continue; }
            if (p_ < t_.size() && t_[p_] == '}') { p_++; return true; }
            return fail("expected ',' or '}' in JSON object");
        }
    }
};

bool asInt(const JValue *v, int &out) {
    if (!v || v->kind != JValue::Number || !v->integral) return false;
    if (v->integer < -2147483647LL || v->integer > 2147483647LL) return false;
    out = (int)v->integer;
    return true;
}

bool readFile(const std::string &path, std::string &out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

bool isDirectory(const std::string &path) {
    struct stat st;
    return stat(path.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

bool endsWith(const std::string &s, const std::string &suffix) {
    return s.size() >= suffix.size() && s.compare(s.size() - suffix.size(), suffix.size(), suffix) == 0;
}

// Integer tokens of a text; false on a token that is not an integer.
bool tokens(const std::string &text, std::vector<long long> &out) {
    std::istringstream is(text);
    std::string tok;
    while (is >> tok) {
        char *end = nullptr;
        long long v = std::strtoll(tok.c_str(), &end, 10);
        if (end == tok.c_str() || *end != '\0') return false;
        out.push_back(v);
    }
    return true;
}

bool sizesOk(long long n1, long long n2, long long n3, long long m) {
    return n1 > 0 && n2 > 0 && n3 > 0 && m >= 0 && n1 <= 64 && n2 <= 64 && n3 <= 64 && m <= 100000;
}

// Reads the rows of one scheme of the given sizes from tokens [p, ...).
bool takeRows(const std::vector<long long> &tk, size_t &p, RawScheme &s) {
    for (int c = 0; c < 3; c++) {
        const size_t need = (size_t)s.m * s.entries(c);
        if (tk.size() - p < need) return false;
        s.rows[c].assign(tk.begin() + p, tk.begin() + p + need);
        p += need;
    }
    return true;
}

}  // namespace

const char *layoutName(TextLayout layout) {
    switch (layout) {
    case TextLayout::FlipGraph: return "flip_graph";
    case TextLayout::Minimizer: return "complexity_minimizer";
    default: return "additions_reducer";
    }
}

namespace {

// One {"index": i, "value": v} term of a reduced expression.
bool reducedTerm(const JValue &t, int &index, int &value) {
    return t.kind == JValue::Object && asInt(t.field("index"), index) && asInt(t.field("value"), value) && index >= 0;
}

// The additions reducer's output (scheme_additions_reducer.cu:395-410, additions_reducer.cuh:304-347)
// expanded back into the scheme it was made from.  Component c has `real` variables (U: n1*n2 entries,
// V: n2*n3, W: the m products) followed by fresh variables, fresh k = value1 * var[index1] +
// value2 * var[index2] over earlier variables; U and V hold one expression per product, W one per
// entry of C over the products, which is transposed back into the m rows of W.
bool expandReduced(const JValue &doc, RawScheme &out, std::string &error) {
    int m = 0;
    if (!asInt(doc.field("m"), m) || m < 0) {
        error = "a reduced scheme needs \"m\"";
        return false;
    }
    out.m = m;
    const char *names[3] = {"u", "v", "w"};
    for (int c = 0; c < 3; c++) {
        const std::string name = names[c];
        const JValue *fresh = doc.field(name + "_fresh"), *exprs = doc.field(name);
        if (!fresh || fresh->kind != JValue::Array || !exprs || exprs->kind != JValue::Array) {
            error = "\"" + name + "\" and \"" + name + "_fresh\" must be arrays";
            return false;
        }
        const int real = c == 2 ? m : out.entries(c);
        const int rows = c == 2 ? out.entries(2) : m;
        if ((int)exprs->items.size() != rows) {
            error = "\"" + name + "\" must hold " + std::to_string(rows) + " expressions";
            return false;
        }
        std::vector<std::vector<int>> var;
        for (int k = 0; k < real; k++) {
            var.emplace_back(real, 0);
            var.back()[k] = 1;
        }
        for (size_t k = 0; k < fresh->items.size(); k++) {
            const JValue &pair = fresh->items[k];
            int i1, v1, i2, v2;
            if (pair.kind != JValue::Array || pair.items.size() != 2 || !reducedTerm(pair.items[0], i1, v1) ||
                !reducedTerm(pair.items[1], i2, v2) || i1 >= (int)var.size() || i2 >= (int)var.size()) {
                error = "fresh variable " + std::to_string(k) + " of \"" + name + "\" is malformed";
                return false;
            }
            std::vector<int> x(real);
            for (int j = 0; j < real; j++) x[j] = v1 * var[i1][j] + v2 * var[i2][j];
            var.push_back(std::move(x));
        }
        std::vector<std::vector<int>> expanded;
        for (int r = 0; r < rows; r++) {
            const JValue &e = exprs->items[r];
            std::vector<int> x(real, 0);
            if (e.kind != JValue::Array) {
                error = "expression " + std::to_string(r) + " of \"" + name + "\" is malformed";
                return false;
            }
            for (const JValue &t : e.items) {
                int index, value;
                if (!reducedTerm(t, index, value) || index >= (int)var.size()) {
                    error = "expression " + std::to_string(r) + " of \"" + name + "\" is malformed";
                    return false;
                }
                for (int j = 0; j < real; j++) x[j] += value * var[index][j];
            }
            expanded.push_back(std::move(x));
        }
        out.rows[c].clear();
        if (c < 2) {
            for (const auto &x : expanded) out.rows[c].insert(out.rows[c].end(), x.begin(), x.end());
        } else {
            for (int t = 0; t < m; t++)
                for (int r = 0; r < rows; r++) out.rows[c].push_back(expanded[r][t]);
        }
    }
    return true;
}

}  // namespace

bool parseSchemeJson(const std::string &text, RawScheme &out, std::string &error) {
    JValue doc;
    JsonReader reader(text);
    if (!reader.document(doc, error)) return false;
    if (doc.kind != JValue::Object) {
        error = "a scheme JSON is an object";
        return false;
    }
    const JValue *n = doc.field("n");
    if (!n || n->kind != JValue::Array || n->items.size() != 3 || !asInt(&n->items[0], out.n[0]) ||
        !asInt(&n->items[1], out.n[1]) || !asInt(&n->items[2], out.n[2]) || out.n[0] <= 0 || out.n[1] <= 0 ||
        out.n[2] <= 0) {
        error = "\"n\" must be an array of three positive integers";
        return false;
    }
    const JValue *z2 = doc.field("z2");
    out.z2 = z2 && z2->kind == JValue::Bool ? (z2->number != 0 ? 1 : 0) : -1;
    if (doc.field("u_fresh")) return expandReduced(doc, out, error);
    const char *names[3] = {"u", "v", "w"};
    int m = -1;
    for (int c = 0; c < 3; c++) {
        const JValue *rows = doc.field(names[c]);
        if (!rows || rows->kind != JValue::Array) {
            error = std::string("\"") + names[c] + "\" must be an array of rows";
            return false;
        }
        if (m < 0) m = (int)rows->items.size();
        if ((int)rows->items.size() != m) {
            error = std::string("\"") + names[c] + "\" has " + std::to_string(rows->items.size()) + " rows, \"u\" has " +
                    std::to_string(m);
            return false;
        }
    }
    const JValue *mv = doc.field("m");
    if (mv) {
        int declared = 0;
        if (!asInt(mv, declared) || declared != m) {
            error = "\"m\" does not match the number of rows (" + std::to_string(m) + ")";
            return false;
        }
    }
    out.m = m;
    for (int c = 0; c < 3; c++) {
        const JValue &rows = *doc.field(names[c]);
        const int e = out.entries(c);
        out.rows[c].clear();
        out.rows[c].reserve((size_t)m * e);
        for (int t = 0; t < m; t++) {
            const JValue &row = rows.items[t];
            if (row.kind != JValue::Array || (int)row.items.size() != e) {
                error = std::string("row ") + std::to_string(t) + " of \"" + names[c] + "\" must hold " + std::to_string(e) +
                        " integers";
                return false;
            }
            for (const JValue &x : row.items) {
                int value = 0;
                if (!asInt(&x, value)) {
                    error = std::string("row ") + std::to_string(t) + " of \"" + names[c] + "\" holds a non-integer";
                    return false;
                }
                out.rows[c].push_back(value);
            }
        }
    }
    return true;
}

bool readSchemeJsonPath(const std::string &path, std::vector<RawScheme> &out, std::string &error) {
    std::vector<std::string> files;
    if (isDirectory(path)) {
        DIR *d = opendir(path.c_str());
        if (!d) {
            error = "unable to open directory \"" + path + "\"";
            return false;
        }
        while (dirent *e = readdir(d)) {
            std::string name = e->d_name;
            if (endsWith(name, ".json")) files.push_back(path + "/" + name);
        }
        closedir(d);
        std::sort(files.begin(), files.end());
        if (files.empty()) {
            error = "no .json files in \"" + path + "\"";
            return false;
        }
    } else {
        files.push_back(path);
    }
    for (const std::string &f : files) {
        std::string text;
        if (!readFile(f, text)) {
            error = "unable to open file \"" + f + "\"";
            return false;
        }
        RawScheme s;
        std::string e;
        if (!parseSchemeJson(text, s, e)) {
            error = f + ": " + e;
            return false;
        }
        out.push_back(std::move(s));
    }
    return true;
}

bool writeTextLayout(const std::vector<RawScheme> &schemes, TextLayout layout, std::ostream &os, std::string &error) {
    auto rows = [&](const RawScheme &s) {
        for (int c = 0; c < 3; c++) {
            const int e = s.entries(c);
            for (int t = 0; t < s.m; t++) {
                for (int j = 0; j < e; j++) os << (j ? " " : "") << s.rows[c][(size_t)t * e + j];
                os << '\n';
            }
        }
    };
    if (schemes.empty()) {
        error = "no schemes to write";
        return false;
    }
    if (layout == TextLayout::Reducer && schemes.size() != 1) {
        error = "the additions_reducer layout holds one scheme (got " + std::to_string(schemes.size()) + ")";
        return false;
    }
    if (layout == TextLayout::Minimizer)
        for (const RawScheme &s : schemes)
            if (s.n[0] != schemes[0].n[0] || s.n[1] != schemes[0].n[1] || s.n[2] != schemes[0].n[2] ||
                s.m != schemes[0].m) {
                error = "the complexity_minimizer layout needs schemes of one size and rank";
                return false;
            }
    if (layout == TextLayout::FlipGraph) os << schemes.size() << '\n';
    const RawScheme &h = schemes[0];
    if (layout == TextLayout::Minimizer)
        os << h.n[0] << ' ' << h.n[1] << ' ' << h.n[2] << ' ' << h.m << ' ' << schemes.size() << '\n';
    for (const RawScheme &s : schemes) {
        if (layout != TextLayout::Minimizer) os << s.n[0] << ' ' << s.n[1] << ' ' << s.n[2] << ' ' << s.m << '\n';
        rows(s);
    }
    return true;
}

bool parseTextLayout(const std::string &text, TextLayout layout, std::vector<RawScheme> &out, std::string &error) {
    std::vector<long long> tk;
    if (!tokens(text, tk)) {
        error = "the text holds a token that is not an integer";
        return false;
    }
    size_t p = 0;
    auto header = [&](RawScheme &s) {
        if (tk.size() - p < 4 || !sizesOk(tk[p], tk[p + 1], tk[p + 2], tk[p + 3])) return false;
        s.n[0] = (int)tk[p]; s.n[1] = (int)tk[p + 1]; s.n[2] = (int)tk[p + 2]; s.m = (int)tk[p + 3];
        p += 4;
        return true;
    };
    const std::string bad = std::string("the text is not in the ") + layoutName(layout) + " layout";
    out.clear();
    if (layout == TextLayout::FlipGraph) {
        if (tk.empty() || tk[0] < 1 || tk[0] > 1000000) { error = bad; return false; }
        const long long count = tk[p++];
        for (long long i = 0; i < count; i++) {
            RawScheme s;
            if (!header(s) || !takeRows(tk, p, s)) { error = bad; return false; }
            out.push_back(std::move(s));
        }
    } else if (layout == TextLayout::Minimizer) {
        RawScheme h;
        if (!header(h) || p >= tk.size() || tk[p] < 1 || tk[p] > 1000000) { error = bad; return false; }
        const long long count = tk[p++];
        for (long long i = 0; i < count; i++) {
            RawScheme s = h;
            if (!takeRows(tk, p, s)) { error = bad; return false; }
            out.push_back(std::move(s));
        }
    } else {
        RawScheme s;
        if (!header(s) || !takeRows(tk, p, s)) { error = bad; return false; }
        out.push_back(std::move(s));
    }
    if (p != tk.size()) {
        error = bad + " (" + std::to_string(tk.size() - p) + " tokens left over)";
        return false;
    }
    return true;
}

std::vector<TextLayout> detectTextLayouts(const std::string &text) {
    std::vector<TextLayout> fits;
    for (TextLayout l : {TextLayout::FlipGraph, TextLayout::Minimizer, TextLayout::Reducer}) {
        std::vector<RawScheme> s;
        std::string e;
        if (parseTextLayout(text, l, s, e)) fits.push_back(l);
    }
    return fits;
}

bool writeSchemeJson(const RawScheme &s, bool zt, std::ostream &os, std::string &error, int bound) {
    int nonzero = 0;
    for (int c = 0; c < 3; c++)
        for (int x : s.rows[c]) {
            if (zt && (x < -bound || x > bound)) {
                error = "coefficient " + std::to_string(x) + (bound == 1 ? " is not ternary" : " exceeds the bound");
                return false;
            }
            nonzero += zt ? (x != 0) : (std::abs(x) % 2);
        }
    os << "{\n";
    os << "    \"n\": [" << s.n[0] << ", " << s.n[1] << ", " << s.n[2] << "],\n";
    os << "    \"m\": " << s.m << ",\n";
    os << "    \"z2\": " << (zt ? "false" : "true") << ",\n";
    os << "    \"complexity\": " << nonzero - 2 * s.m - s.entries(2) << ",\n";
    const char *names[3] = {"u", "v", "w"};
    for (int c = 0; c < 3; c++) {
        const int e = s.entries(c);
        os << "    \"" << names[c] << "\": [\n";
        for (int t = 0; t < s.m; t++) {
            os << "        [";
            for (int j = 0; j < e; j++) {
                const int x = s.rows[c][(size_t)t * e + j];
                os << (j ? ", " : "") << (zt ? x : std::abs(x) % 2);
            }
            os << "]" << (t < s.m - 1 ? "," : "") << "\n";
        }
        os << "    ]" << (c < 2 ? ",\n" : "\n");
    }
    os << "}\n";
    return true;
}

bool isJsonInput(const std::string &path) {
    if (isDirectory(path)) return true;
    std::ifstream f(path);
    char ch = 0;
    while (f.get(ch))
        if (!std::isspace((unsigned char)ch)) return ch == '{';
    return false;
}

bool openSchemeInput(const std::string &path, TextLayout layout, std::stringstream &out, std::string &error) {
    if (!isJsonInput(path)) {
        std::string text;
        if (!readFile(path, text)) {
            error = "Unable to open file \"" + path + "\"";
            return false;
        }
        out.str(text);
        return true;
    }
    std::vector<RawScheme> schemes;
    if (!readSchemeJsonPath(path, schemes, error)) return false;
    std::ostringstream os;
    if (!writeTextLayout(schemes, layout, os, error)) return false;
    out.str(os.str());
    return true;
}

}  // namespace fgcli
