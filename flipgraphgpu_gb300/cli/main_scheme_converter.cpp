// scheme_converter: converts scheme files between the JSON the executables
// save and the text layouts they read (flip_graph, complexity_minimizer,
// additions_reducer), so that a run can be resumed from its own output by the
// reference's executables too.  No counterpart in the reference, which writes
// JSON (scheme_z2.cu:1327-1364, scheme_integer.cu:1247-1274) and reads only
// text (scheme_z2.cu:72-96, scheme_integer.cu:81-107).  Host only: no device
// work.
//
//   scheme_converter -i IN -o OUT [--to auto|text|json] [--layout auto|flip_graph|
//                    complexity_minimizer|additions_reducer] [--ring auto|ZT|Z2]
//
// JSON input (one file, or a directory of *.json read in name order) becomes
// text in the chosen layout (flip_graph by default).  Text input (layout
// detected from its token counts unless given) becomes JSON: one scheme is
// written to OUT, several to the directory OUT as
// <index, 6 digits>_<sorted size>_m<rank>_c<complexity>_<n1>x<n2>x<n3>_<ring>.json,
// so that reading the directory back (name order) keeps the input order.
// The ring decides how JSON is written: Z2 writes |value| mod 2, ZT and ZB the
// values (bound 1 and 2); "auto" takes a JSON input's "z2" key, and ZT for text
// (the reference's default build), ZB when an integer entry has magnitude 2.  Exit status 0 on success, 1 on any error (message on stderr).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <sys/stat.h>

#include "common.h"
#include "scheme_io.h"

using namespace fgcli;

namespace {

bool readAll(const std::string &path, std::string &out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

int fail(const std::string &msg) {
    std::cerr << "scheme_converter: " << msg << std::endl;
    return 1;
}

// The zero-padded index leads the name, so that name order is input order.
std::string jsonName(const RawScheme &s, int index, bool zt, int complexity, const std::string &ringOverride) {
    char idx[16];
    std::snprintf(idx, sizeof idx, "%06d", index);
    return std::string(idx) + "_" + key(s.n[0], s.n[1], s.n[2]) + "_m" + std::to_string(s.m) + "_c" +
           std::to_string(complexity) + "_" + key(s.n[0], s.n[1], s.n[2], false) + "_" +
           (ringOverride.empty() ? ringName(zt) : ringOverride) + ".json";
}

int complexityOf(const RawScheme &s, bool zt) {
    int nonzero = 0;
    for (int c = 0; c < 3; c++)
        for (int x : s.rows[c]) nonzero += zt ? (x != 0) : (x % 2 != 0);
    return nonzero - 2 * s.m - s.entries(2);
}

}  // namespace

int main(int argc, char *argv[]) {
    ArgParser parser("scheme_converter", "Convert matrix multiplication schemes between JSON and the text layouts");
    parser.add("-i", ArgType::String, "PATH", "input: a scheme JSON file, a directory of them, or a text file", "");
    parser.add("-o", ArgType::String, "PATH", "output file (or directory for several JSON schemes)", "");
    parser.add("--to", ArgType::String, "auto|text|json", "output format (auto: the other one)", "auto");
    parser.add("--layout", ArgType::String, "auto|flip_graph|complexity_minimizer|additions_reducer",
               "text layout written, or read (auto: flip_graph when writing, detected when reading)", "auto");
    parser.add("--ring", ArgType::String, "auto|ZT|Z2|ZB", "ring of the JSON written (ZB: integers, |c| <= 2)", "auto");
    if (!parser.parse(argc, argv)) return 0;

    const std::string in = parser.get("-i"), out = parser.get("-o"), to = parser.get("--to");
    const std::string layoutArg = parser.get("--layout"), ring = parser.get("--ring");
    if (in.empty() || out.empty()) return fail("-i and -o are required");
    if (to != "auto" && to != "text" && to != "json") return fail("unknown --to \"" + to + "\"");
    if (ring != "auto" && ring != "ZT" && ring != "Z2" && ring != "ZB") return fail("unknown --ring \"" + ring + "\"");
    bool layoutGiven = layoutArg != "auto";
    TextLayout layout = TextLayout::FlipGraph;
    if (layoutArg == "complexity_minimizer") layout = TextLayout::Minimizer;
    else if (layoutArg == "additions_reducer") layout = TextLayout::Reducer;
    else if (layoutArg != "auto" && layoutArg != "flip_graph") return fail("unknown --layout \"" + layoutArg + "\"");

    const bool jsonIn = isJsonInput(in);
    std::vector<RawScheme> schemes;
    std::string error;
    if (jsonIn) {
        if (!readSchemeJsonPath(in, schemes, error)) return fail(error);
    } else {
        std::string text;
        if (!readAll(in, text)) return fail("unable to open file \"" + in + "\"");
        if (!layoutGiven) {
            std::vector<TextLayout> fits = detectTextLayouts(text);
            if (fits.empty()) return fail("the text is in none of the layouts");
            if (fits.size() > 1) {
                std::string names;
                for (TextLayout l : fits) names += std::string(names.empty() ? "" : ", ") + layoutName(l);
                return fail("the text reads in several layouts (" + names + "); give --layout");
            }
            layout = fits[0];
        }
        if (!parseTextLayout(text, layout, schemes, error)) return fail(error);
    }

    const bool toJson = to == "json" || (to == "auto" && !jsonIn);
    if (!toJson) {
        std::ofstream f(out);
        if (!f) return fail("unable to write \"" + out + "\"");
        if (!writeTextLayout(schemes, layout, f, error)) return fail(error);
        std::cout << "Wrote " << schemes.size() << " scheme(s) to \"" << out << "\" (" << layoutName(layout)
                  << " layout)" << std::endl;
        return 0;
    }
    if (schemes.size() > 1) mkdir(out.c_str(), 0755);
    for (size_t i = 0; i < schemes.size(); i++) {
        const RawScheme &s = schemes[i];
        const bool zt = ring == "ZT" || ring == "ZB" || (ring == "auto" && s.z2 != 1);
        // auto: an integer scheme with an entry of magnitude 2 is written as the |c| <= 2 ring
        int maxAbs = 0;
        for (int c = 0; c < 3; c++)
            for (int x : s.rows[c]) maxAbs = std::max(maxAbs, std::abs(x));
        const bool zb = ring == "ZB" || (ring == "auto" && zt && maxAbs == 2);
        const std::string path =
            schemes.size() == 1 ? out : out + "/" + jsonName(s, (int)i, zt, complexityOf(s, zt), zb ? "ZB" : "");
        std::ofstream f(path);
        if (!f) return fail("unable to write \"" + path + "\"");
        if (!writeSchemeJson(s, zt, f, error, zb ? 2 : 1)) return fail("scheme " + std::to_string(i) + ": " + error);
    }
    std::cout << "Wrote " << schemes.size() << " scheme(s) to \"" << out << "\" (JSON)" << std::endl;
    return 0;
}
