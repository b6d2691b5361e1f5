"""Flag grammar of the executables (no GPU needed: parsing fails before any device work)."""
import os
import platform
import subprocess

import pytest

fg = pytest.importorskip("flipgraphgpu_gb300")
BIN = os.path.join(os.path.dirname(fg.__file__), "_lib", platform.machine())


def run(*args):
    exe = os.path.join(BIN, args[0])
    if not os.path.exists(exe):
        pytest.skip("executables not built")
    r = subprocess.run([exe, *args[1:]], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=60)
    return r.returncode, r.stdout, r.stderr


def test_help_lists_reference_flags():
    rc, out, _ = run("flip_graph", "--help")
    assert rc == 0
    for flag in ["-n1 INT", "[--schemes 1024]", "[--max-iterations 10000]", "[--path schemes]", "[--input-path null]",
                 "[--block-size 32]", "[--expand-probability 0.01]", "[--reduce-probability 0.0]",
                 "[--sandwiching-probability 0.0]", "[--basis-probability 0.0]", "[--resize-probability 0.2]",
                 "[--plus-iterations 8000]", "[--log-period 0]", "[--seed 0]"]:
        assert flag in out, flag
    rc, out, _ = run("complexity_minimizer", "--help")
    for flag in ["[--schemes 1024]", "[--max-iterations 10000]", "--input-path PATH", "[--target-complexity 0]",
                 "[--max-no-improvements 3]"]:
        assert flag in out, flag
    rc, out, _ = run("additions_reducer", "--help")
    for flag in ["-i PATH", "[-o schemes/additions_reduced]", "[--count 32]", "[--schemes-count 1]",
                 "[--start-additions 0]", "[--max-flips 0]", "[--max-no-improvements 3]"]:
        assert flag in out, flag


def test_grammar_errors():
    rc, _, err = run("flip_graph", "-n1", "3", "-n2")
    assert "Invalid number of arguments" in err
    rc, _, err = run("flip_graph", "-n1", "3", "-n2", "3", "-n3", "x3")
    assert 'value for arg "-n3" is not natural (x3)' in err
    rc, _, err = run("flip_graph", "-n1", "3", "-n2", "3", "-n3", "3", "--expand-probability", "0.1.2")
    assert 'is not real (0.1.2)' in err
    rc, _, err = run("flip_graph", "-n1", "3", "-n2", "3", "-n3", "3", "--bogus", "1")
    assert 'unknown argument "--bogus"' in err
    rc, _, err = run("flip_graph", "-n1", "3", "-n3", "3")
    assert 'no value for argument "-n2"' in err


def test_size_limits():
    rc, out, _ = run("flip_graph", "-n1", "9", "-n2", "8", "-n3", "2")
    assert "Error sizes, please increase MAX_MATRIX_ELEMENTS (now: 64)" in out and rc == 0
    rc, out, _ = run("flip_graph", "-n1", "8", "-n2", "8", "-n3", "8")
    assert "Error sizes, please increase MAX_RANK (now: 350)" in out and rc == 0


def test_missing_input_files():
    rc, out, _ = run("complexity_minimizer", "--input-path", "/nonexistent/x.txt")
    assert 'Unable to open file "/nonexistent/x.txt"' in out and rc == 255
    rc, out, _ = run("additions_reducer", "-i", "/nonexistent/x.txt")
    assert 'Unable to open file "/nonexistent/x.txt"' in out and rc == 255


def test_ring_and_input_checks():
    rc, _, err = run("flip_graph", "-n1", "3", "-n2", "3", "-n3", "3", "--ring", "ZQ")
    assert 'unknown ring "ZQ"' in err
    rc, out, _ = run("flip_graph", "-n1", "3", "-n2", "3", "-n3", "3", "--ring", "ZB", "--input-path", "x.json")
    assert "the ZB ring starts from the naive scheme" in out and rc == 255
    rc, out, _ = run("flip_graph", "-n1", "3", "-n2", "3", "-n3", "3", "--input-path", "/nonexistent/x.txt",
                     "--ring", "Z2")
    assert 'Unable to open file "/nonexistent/x.txt"' in out and rc == 255
    rc, out, _ = run("flip_graph", "--help")
    for flag in ["[--gauss-probability 0.0]", "[--ternary-sandwiching 0]", "[--max-launches 0]"]:
        assert flag in out, flag


def test_json_input_errors(tmp_path):
    bad = tmp_path / "bad.json"
    bad.write_text('{"n": [2, 2, 2], "u": [[1, 0, 0, 0]], "v": [], "w": []}')
    rc, out, _ = run("complexity_minimizer", "--input-path", str(bad))
    assert '"v" has 0 rows' in out and rc == 255
    empty = tmp_path / "empty"
    empty.mkdir()
    rc, out, _ = run("additions_reducer", "-i", str(empty))
    assert "no .json files" in out and rc == 255


def test_ternary_input_flags_coefficients_outside_the_ring(tmp_path):
    """A ZT text input with a coefficient outside {-1, 0, 1} is reported while it is read
    (Addition::set, addition.cu:41-60), before any device work."""
    import gzip
    from helpers import GOLDEN
    tokens = gzip.open(os.path.join(GOLDEN, "input_zt_333.txt.gz"), "rt").read().split()
    head, body = tokens[:4], tokens[4:]
    body[0] = "2"
    src = tmp_path / "two.txt"
    src.write_text("1\n" + " ".join(head) + "\n" + " ".join(body) + "\n")
    rc, out, _ = run("flip_graph", "-n1", "3", "-n2", "3", "-n3", "3", "--input-path", str(src), "--ring", "ZT",
                     "--schemes", "32", "--max-iterations", "10", "--max-launches", "1", "--path", str(tmp_path / "o"))
    assert "invalid set (0, 2)" in out


def test_max_flips_needs_a_stream_per_scheme(tmp_path):
    """--max-flips flips scheme s with reducer s's stream (flipSchemesKernel), so the
    executable refuses more schemes than reducers before any device work."""
    import gzip
    from helpers import GOLDEN
    src = tmp_path / "in.txt"
    src.write_text(gzip.open(os.path.join(GOLDEN, "input_zt_333.txt.gz"), "rt").read())
    rc, out, _ = run("additions_reducer", "-i", str(src), "-o", str(tmp_path), "--count", "4", "--schemes-count", "8",
                     "--max-flips", "5")
    assert "- max flips: 5" in out
    assert "--schemes-count must not exceed --count" in out and rc == 255
