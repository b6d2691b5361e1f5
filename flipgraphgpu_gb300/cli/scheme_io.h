// Scheme files across the executables: the JSON every executable saves
// (SchemeZ2::save / SchemeInteger::save, scheme_z2.cu:1327-1364,
// scheme_integer.cu:1247-1274) read back as input, and the three text
// layouts the reference's executables read:
//
//   flip_graph            "count", then per scheme "n1 n2 n3 m" and its rows
//                         (flip_graph.cu:201-224)
//   complexity_minimizer  "n1 n2 n3 m count", then per scheme its rows
//                         (complexity_minimizer.cu:23-35)
//   additions_reducer     "n1 n2 n3 m" and the rows of one scheme
//                         (scheme_additions_reducer.cu:29-90)
//
// Rows are U's m rows of n1*n2 entries, then V's (n2*n3), then W's (n3*n1),
// W transposed as in the JSON.  The reference writes JSON and reads only
// text, so resuming a run from its own output needs a conversion; here every
// executable accepts a JSON file or a directory of JSON files wherever it
// takes a text file, and `scheme_converter` converts both ways.
#pragma once
#include <iosfwd>
#include <sstream>
#include <string>
#include <vector>

namespace fgcli {

// One scheme as the integers of its file, before any ring interpretation.
struct RawScheme {
    int n[3] = {0, 0, 0};
    int m = 0;
    std::vector<int> rows[3];  // component c: m rows of n[c] * n[(c + 1) % 3] entries
    int z2 = -1;               // the JSON's "z2" key: 1 true, 0 false, -1 absent (text input)
    int entries(int c) const { return n[c] * n[(c + 1) % 3]; }
};

enum class TextLayout { FlipGraph, Minimizer, Reducer };

// Parses one scheme JSON document (keys n, u, v, w; m, z2 and complexity are
// optional, m must match the rows, complexity is not read; any key order and
// whitespace).  The additions reducer's output (u_fresh, v_fresh, w_fresh and
// sparse expressions) is expanded back into the scheme it was made from.  False with `error` set
// on malformed JSON, missing keys or rows of the wrong length.
bool parseSchemeJson(const std::string &text, RawScheme &out, std::string &error);

// Reads `path`: a scheme JSON file, or a directory whose *.json files are read
// in name order.  False with `error` set when nothing could be read.
bool readSchemeJsonPath(const std::string &path, std::vector<RawScheme> &out, std::string &error);

// Writes schemes in one of the executables' text layouts.  The minimizer layout
// needs one common size and rank, the reducer layout exactly one scheme.
bool writeTextLayout(const std::vector<RawScheme> &schemes, TextLayout layout, std::ostream &os, std::string &error);

// Parses text in a given layout into raw schemes (no ring interpretation).
bool parseTextLayout(const std::string &text, TextLayout layout, std::vector<RawScheme> &out, std::string &error);

// The layouts a text parses in completely (every token consumed).
std::vector<TextLayout> detectTextLayouts(const std::string &text);

// True when the path is a directory or a file whose first non-space character is '{'.
bool isJsonInput(const std::string &path);

// Input for an executable that reads `layout`: a text file is passed through
// unchanged, JSON input is rewritten into `layout`.  False with `error` set
// when the path cannot be read or does not fit the layout.
bool openSchemeInput(const std::string &path, TextLayout layout, std::stringstream &out, std::string &error);

const char *layoutName(TextLayout layout);

// The scheme JSON exactly as SchemeZ2::save / SchemeInteger::save write it,
// from raw integers: Z2 writes |value| mod 2, the integer rings write the
// values, which must lie in [-bound, bound] (1: ZT, 2: the |c| <= 2 ring).
// Complexity = nonzero entries - 2m - n3*n1 (getComplexity).
bool writeSchemeJson(const RawScheme &s, bool zt, std::ostream &os, std::string &error, int bound = 1);

}  // namespace fgcli
