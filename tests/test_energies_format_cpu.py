"""The energy-history text formats against the C and C++ libraries that write
them in the reference (src/fields.h:722-763): energies.txt through a
std::ostream at its default precision (energy_line), and the stdout line of
printf("%d %f %e %e\\n") (stdout_line), which is the format of the
reference's gold files.  A small g++ program prints both for the same values.
The particle and field dump lines are checked against C printf the same way."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from cabanapic_gb300 import energies as E
from conftest import gold_path

_CPP = r"""
#include <cstdio>
#include <cstdlib>
#include <iostream>
int main(int argc, char** argv) {
  // stdin: step time e b per line; stdout: the ostream line, then the printf line
  int step; double t, e, b;
  while (std::scanf("%d %lf %lf %lf", &step, &t, &e, &b) == 4) {
    std::cout << step << " " << t << " " << e << " " << b << std::endl;
    std::printf("%d %f %e %e\n", step, t, e, b);
    std::fflush(stdout);
    // the ES_FIELD_SOLVER build: no B token
    std::cout << step << " " << t << " " << e << std::endl;
    std::printf("%d %f %e\n", step, t, e);
    std::fflush(stdout);
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def cpp_format(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("fmt")
    src, exe = d / "fmt.cpp", d / "fmt"
    src.write_text(_CPP)
    subprocess.run([gxx, "-O1", "-o", str(exe), str(src)], check=True)

    def run(rows):
        inp = "".join(f"{s} {t!r} {e!r} {b!r}\n" for s, t, e, b in rows)
        out = subprocess.run([str(exe)], input=inp, capture_output=True, text=True, check=True).stdout
        lines = out.splitlines()
        return lines[0::4], lines[1::4], lines[2::4], lines[3::4]

    return run


def _rows():
    rng = np.random.default_rng(5)
    mags = 10.0 ** rng.uniform(-120, 120, 300)
    vals = list(mags * rng.choice([-1, 1], 300)) + [0.0, 1.0, 0.1, 1e-5, 123456.5, 1234567.0, 0.0001,
                                                     9.9999995e-5, 2.5e100, 1e-300]
    rows = []
    for i, v in enumerate(vals):
        rows.append((i, 0.019549 * i, float(v), float(abs(v) * 0.37 + 1e-20)))
    return rows


def test_ostream_and_printf_lines_match_the_c_libraries(cpp_format):
    rows = _rows()
    ostream, printf, ostream_es, printf_es = cpp_format(rows)
    assert len(ostream) == len(rows) == len(printf) == len(ostream_es) == len(printf_es)
    for (s, t, e, b), lo, lp, leo, lep in zip(rows, ostream, printf, ostream_es, printf_es):
        assert E.energy_line(s, t, e, b) == lo
        assert E.stdout_line(s, t, e, b) == lp
        assert E.energy_line(s, t, e) == leo
        assert E.stdout_line(s, t, e) == lep


def test_oracle_formatter_agrees_with_the_product_formatter(cpp_format):
    """The oracle keeps its own restatement of the energies.txt line (test
    infrastructure does not import the product's formatter); both must give
    the same text, here on the gold values and on the C-checked rows."""
    from oracle import energy_rule
    g = np.loadtxt(gold_path("double"))
    rows = [(int(r[0]), r[1], r[2], r[3]) for r in g] + _rows()
    for s, t, e, b in rows:
        assert energy_rule.format_energy_line(s, t, e, b) == E.energy_line(s, t, e, b)


@pytest.mark.parametrize("kind", ["float", "double"])
def test_stdout_line_reproduces_the_gold_files(kind):
    lines = open(gold_path(kind)).read().splitlines()
    assert len(lines) == 6000
    for ln in lines:
        s, t, e, b = ln.split(" ")
        assert E.stdout_line(int(s), float(t), float(e), float(b)) == ln


def test_history_in_either_format_passes_the_rule_against_gold(tmp_path):
    from cabanapic_gb300 import decks
    g = np.loadtxt(gold_path("double"))
    dt = decks.two_stream_em(precision=8).dt
    for fmt in (False, True):
        path = tmp_path / f"e{int(fmt)}.txt"
        E.write_history(str(path), g[:, 2:4], dt, first_step=0, stdout_format=fmt)
        (e_ok, e_err, _), (b_ok, b_err, _) = E.two_stream_em_rule(gold_path("double"), str(path))
        assert e_ok and b_ok and e_err < 1e-5 and b_err < 1e-5
    # the stdout format with the deck's dt rewrites the gold file byte for byte
    assert open(tmp_path / "e1.txt").read() == open(gold_path("double")).read()


def test_pic_dump_energies_writes_the_file_and_echoes_the_stdout_line(tmp_path, capsys):
    """pic.dump_energies over a stand-in solver (the energies come from the
    device in real runs): truncates at step 0, appends after, and prints the
    reference's stdout line."""
    torch = pytest.importorskip("torch")
    from cabanapic_gb300 import pic

    vals = {0: (8.973809e-13, 8.449903e-15), 1: (3.455599e-12, 1.326642e-13), 2: (7.283853e-12, 6.504499e-13)}

    class Solver:
        step = 0

        def energies_async(self, fields, nx, ny, nz, ng):
            return torch.tensor(vals[self.step], dtype=torch.float64)

    path = tmp_path / "energies.txt"
    path.write_text("stale\n")
    s = Solver()
    dt = 0.0195487
    for k in range(3):
        s.step = k
        pic.dump_energies(s, None, k, k * dt, 0, 0, 0, 4, 4, 4, 1, path=str(path))
    assert path.read_text().splitlines() == [E.energy_line(k, k * dt, *vals[k]) for k in range(3)]
    assert capsys.readouterr().out.splitlines() == [E.stdout_line(k, k * dt, *vals[k]) for k in range(3)]
    s.step = 0
    pic.dump_energies(s, None, 0, 0.0, 0, 0, 0, 4, 4, 4, 1, path=str(path), echo=False)
    assert path.read_text().splitlines() == [E.energy_line(0, 0.0, *vals[0])]
    assert capsys.readouterr().out == ""


def test_pic_dump_energies_with_an_es_solver(tmp_path, capsys):
    """With an ES solver (the reference's ES_FIELD_SOLVER build) dump_energies
    writes and prints `step time E` only (src/fields.h:751-759)."""
    pytest.importorskip("torch")
    from cabanapic_gb300 import pic

    vals = [4.25e-3, 3.5e-3]

    class Solver(pic.ESFieldSolver1D):
        step = 0

        def e_energy(self, fields, px, py, pz, nx, ny, nz, ng, *, stream=None):
            return vals[self.step]

    path = tmp_path / "energies.txt"
    s = Solver()
    dt = 0.0195487
    for k in range(2):
        s.step = k
        e, b = pic.dump_energies(s, None, k, k * dt, 0, 0, 0, 32, 1, 1, 1, path=str(path))
        assert (e, b) == (vals[k], None)
    assert path.read_text().splitlines() == [E.energy_line(k, k * dt, vals[k]) for k in range(2)]
    assert capsys.readouterr().out.splitlines() == [E.stdout_line(k, k * dt, vals[k]) for k in range(2)]
    assert all(len(l.split(" ")) == 3 for l in path.read_text().splitlines())


_CPP_PAIRS = r"""
#include <cstdio>
int main() {
  // stdin: pairs of floats; stdout: the particle dump's "%e  %e " per pair,
  // a newline, then the field dump's "%e %e\n" per pair
  static float v[4096];
  int n = 0;
  while (n < 4096 && std::scanf("%f", &v[n]) == 1) ++n;
  for (int i = 0; i + 1 < n; i += 2) std::printf("%e  %e ", v[i], v[i + 1]);
  std::printf("\n");
  for (int i = 0; i + 1 < n; i += 2) std::printf("%e %e\n", v[i], v[i + 1]);
  return 0;
}
"""


def test_dump_pairs_match_c_printf(tmp_path):
    """The particle and field dump lines (fprintf "%e  %e " and "%e %e\\n" of
    real_t values in the reference) from FP32 values, against C printf."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    from cabanapic_gb300 import pic
    src, exe = tmp_path / "pairs.cpp", tmp_path / "pairs"
    src.write_text(_CPP_PAIRS)
    subprocess.run([gxx, "-O1", "-o", str(exe), str(src)], check=True)
    rng = np.random.default_rng(9)
    v = (rng.standard_normal(400) * 10.0 ** rng.uniform(-30, 30, 400)).astype(np.float32)
    v[:4] = [0.0, -0.0, 1.0, -3.5]
    inp = " ".join(repr(float(x)) for x in v)
    out = subprocess.run([str(exe)], input=inp, capture_output=True, text=True, check=True).stdout
    expect = pic._fmt_pairs(v, "  ", " ") + "\n" + pic._fmt_pairs(v, " ", "\n")
    assert out == expect
