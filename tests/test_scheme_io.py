"""Scheme files: the JSON the executables save, read back as input, and the
scheme_converter executable (host only, so these run without a GPU).

* Every JSON the reference's executables saved (tests/golden/cli_*) converts
  to text and back to byte-identical JSON, in every layout it fits.
* The reference's own text inputs are recognised in their layouts and survive
  text -> JSON -> text token for token.
* The additions reducer's output (fresh variables, sparse expressions) expands
  back into exactly the scheme the reducer was given.
* Malformed inputs are rejected with a message and a non-zero exit status.
"""
import glob
import gzip
import json
import os
import platform
import subprocess

import pytest

from helpers import GOLDEN

fg = pytest.importorskip("flipgraphgpu_gb300")
BIN = os.path.join(os.path.dirname(fg.__file__), "_lib", platform.machine())
CONV = os.path.join(BIN, "scheme_converter")

REFERENCE_JSON = sorted(p for p in glob.glob(os.path.join(GOLDEN, "cli_*", "*.json"))
                        if "cli_additions_reducer" not in p)
REDUCED_JSON = sorted(glob.glob(os.path.join(GOLDEN, "cli_additions_reducer", "*.json")))


def conv(*args, ok=True):
    if not os.path.exists(CONV):
        pytest.skip("executables not built")
    r = subprocess.run([CONV, *map(str, args)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=60)
    if ok:
        assert r.returncode == 0, r.stderr
    return r


def unpack(name, dst):
    with gzip.open(os.path.join(GOLDEN, name + ".gz"), "rb") as f:
        data = f.read()
    path = os.path.join(dst, name)
    with open(path, "wb") as o:
        o.write(data)
    return path


def test_reference_json_round_trips_through_every_layout(tmp_path):
    assert len(REFERENCE_JSON) >= 40
    for src in REFERENCE_JSON:
        ring = "Z2" if json.load(open(src))["z2"] else "ZT"
        for layout in ("flip_graph", "complexity_minimizer", "additions_reducer"):
            txt, back = tmp_path / "s.txt", tmp_path / "s.json"
            conv("-i", src, "-o", txt, "--layout", layout)
            conv("-i", txt, "-o", back, "--layout", layout, "--ring", ring)
            assert open(src).read() == back.read_text(), (src, layout)


def test_ring_is_taken_from_the_json(tmp_path):
    for src in REFERENCE_JSON[:40]:
        txt, back = tmp_path / "s.txt", tmp_path / "s.json"
        conv("-i", src, "-o", txt)
        conv("-i", txt, "-o", back, "--to", "json")  # text input: ZT unless told
        conv("-i", src, "-o", back, "--to", "json")   # JSON input: its own "z2" key
        assert open(src).read() == back.read_text(), src


def test_directory_input_in_name_order(tmp_path):
    d = os.path.join(GOLDEN, "cli_flip_graph_moves")
    names = sorted(x for x in os.listdir(d) if x.endswith(".json"))
    txt = tmp_path / "all.txt"
    conv("-i", d, "-o", txt)
    tokens = txt.read_text().split()
    assert int(tokens[0]) == len(names)
    first = json.load(open(os.path.join(d, names[0])))
    assert [int(x) for x in tokens[1:5]] == first["n"] + [first["m"]]
    out = tmp_path / "out"
    conv("-i", txt, "-o", out, "--ring", "Z2")
    got = sorted(os.listdir(out))
    assert len(got) == len(names)
    for i, name in enumerate(names):
        mine = [g for g in got if g.startswith(f"{i:06d}_")]
        assert len(mine) == 1
        assert open(os.path.join(d, name)).read() == open(os.path.join(out, mine[0])).read()


@pytest.mark.parametrize("name,layout", [("input_zt_333.txt", "additions_reducer"),
                                         ("input_z2_333.txt", "additions_reducer"),
                                         ("input_minimizer_z2_333.txt", "complexity_minimizer")])
def test_reference_text_inputs(tmp_path, name, layout):
    src = unpack(name, str(tmp_path))
    js = tmp_path / "j"
    conv("-i", src, "-o", js)  # layout detected
    r = conv("-i", src, "-o", tmp_path / "x.txt", "--to", "text")
    assert layout in r.stdout
    back = tmp_path / "back.txt"
    conv("-i", js, "-o", back, "--layout", layout)  # a file, or a directory for several schemes
    assert open(src).read().split() == back.read_text().split()


def test_reduced_schemes_expand_to_the_reducers_input(tmp_path):
    assert REDUCED_JSON
    want = gzip.open(os.path.join(GOLDEN, "input_zt_333.txt.gz"), "rt").read().split()
    for src in REDUCED_JSON:
        txt = tmp_path / "r.txt"
        conv("-i", src, "-o", txt, "--layout", "additions_reducer")
        assert txt.read_text().split() == want, src
    # and as a directory, for the minimizer
    conv("-i", os.path.dirname(REDUCED_JSON[0]), "-o", tmp_path / "all.txt", "--layout", "complexity_minimizer")
    got = (tmp_path / "all.txt").read_text().split()
    assert got[:5] == want[:4] + [str(len(REDUCED_JSON))]
    body = want[4:]
    assert got[5:] == body * len(REDUCED_JSON)


def test_rejects_malformed_input(tmp_path):
    good = json.load(open(REFERENCE_JSON[0]))
    cases = {
        "trailing": json.dumps(good) + " x",
        "no_n": json.dumps({k: v for k, v in good.items() if k != "n"}),
        "short_row": json.dumps(dict(good, u=[good["u"][0][:-1]] + good["u"][1:])),
        "rank": json.dumps(dict(good, m=good["m"] + 1)),
        "float": json.dumps(dict(good, v=[[0.5] * len(good["v"][0])] + good["v"][1:])),
        "rows": json.dumps(dict(good, w=good["w"][:-1])),
        "syntax": json.dumps(good)[:-5],
        "reduced": json.dumps(dict(json.load(open(REDUCED_JSON[0])), u_fresh=[[{"index": 999, "value": 1}] * 2])),
    }
    for name, text in cases.items():
        p = tmp_path / f"{name}.json"
        p.write_text(text)
        r = conv("-i", p, "-o", tmp_path / "o.txt", ok=False)
        assert r.returncode == 1 and "scheme_converter:" in r.stderr, name
    # A coefficient outside {-1, 0, 1} cannot be written as a ternary scheme.
    bad = dict(good, u=[[2] * len(good["u"][0])] + good["u"][1:])
    p = tmp_path / "two.json"
    p.write_text(json.dumps(bad))
    r = conv("-i", p, "-o", tmp_path / "o.json", "--to", "json", "--ring", "ZT", ok=False)
    assert r.returncode == 1 and "not ternary" in r.stderr
    # Z2 keeps the residue mod 2.
    conv("-i", p, "-o", tmp_path / "o.json", "--to", "json", "--ring", "Z2")
    assert json.load(open(tmp_path / "o.json"))["u"][0] == [0] * len(good["u"][0])
    # Text that is no layout, and text that fits several, need a decision.
    (tmp_path / "junk.txt").write_text("1 2 3")
    assert conv("-i", tmp_path / "junk.txt", "-o", tmp_path / "o.json", ok=False).returncode == 1
    (tmp_path / "empty").mkdir()
    r = conv("-i", tmp_path / "empty", "-o", tmp_path / "o.txt", ok=False)
    assert r.returncode == 1 and "no .json files" in r.stderr


def test_layout_constraints(tmp_path):
    d = os.path.join(GOLDEN, "cli_flip_graph_moves")  # several sizes
    r = conv("-i", d, "-o", tmp_path / "o.txt", "--layout", "complexity_minimizer", ok=False)
    assert r.returncode == 1 and "one size and rank" in r.stderr
    r = conv("-i", d, "-o", tmp_path / "o.txt", "--layout", "additions_reducer", ok=False)
    assert r.returncode == 1 and "holds one scheme" in r.stderr
