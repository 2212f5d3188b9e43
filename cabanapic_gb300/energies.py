"""energies.txt: the reference's energy-history format and its comparison rule.

energy_line / write_history produce the `step time E B` lines that
dump_energies writes to energies.txt (src/fields.h:722-763: a std::ostream at
its default 6-significant-digit precision, one line per step, steps from 1);
stdout_line is the line it prints to stdout at the same time (printf
"%d %f %e %e"), the format of the reference's gold energy files.  compare_files applies the rule of
the reference's regression test (tests/energy_comparison/compare_energies.h:
69-106, 135-362, as called by 2stream-em.cxx:45-70): skip N lines, then for M
lines sum the masked tokens (bit k selects token k, token 0 = step) and
compare with a relative tolerance, or an absolute one of 2 double epsilons
when the smaller value is below 10 epsilons.
"""
from __future__ import annotations

import sys
from typing import List, Sequence, Tuple

EPS = sys.float_info.epsilon


def _fmt(v: float) -> str:
    s = f"{v:.6g}"
    if "e" in s:  # at least two exponent digits, as printf %g / ostream
        mant, exp = s.split("e")
        digits = exp[1:].lstrip("0") or "0"
        s = f"{mant}e{exp[0]}{digits.zfill(2)}"
    return s


def energy_line(step: int, time: float, e: float, b: float = None) -> str:
    """The energies.txt line; b=None gives the ES solvers' `step time E`
    line (fields.h:751-759 writes B only for the EM solver)."""
    if b is None:
        return f"{step} {_fmt(time)} {_fmt(e)}"
    return f"{step} {_fmt(time)} {_fmt(e)} {_fmt(b)}"


def stdout_line(step: int, time: float, e: float, b: float = None) -> str:
    """printf("%d %f %e %e") of the EM solver, printf("%d %f %e") when b is
    None (the ES solvers)."""
    if b is None:
        return f"{step} {time:f} {e:e}"
    return f"{step} {time:f} {e:e} {b:e}"


def history_lines(energies: Sequence[Sequence[float]], dt: float, first_step: int = 1,
                  stdout_format: bool = False) -> List[str]:
    fmt = stdout_line if stdout_format else energy_line
    return [fmt(first_step + i, (first_step + i) * dt, float(r[0]), float(r[1]))
            for i, r in enumerate(energies)]


def write_history(path: str, energies, dt: float, first_step: int = 1, stdout_format: bool = False) -> None:
    with open(path, "w") as fh:
        for line in history_lines(energies, dt, first_step, stdout_format):
            fh.write(line + "\n")


def _relative_or_absolute(a: float, b: float, tol: float) -> Tuple[bool, float]:
    if abs(min(a, b)) < 10 * EPS:
        err = abs(a - b)
        return err < 2 * EPS, err
    err = abs(a - b) / min(a, b)
    return err < tol, err


def compare_files(file_a, file_b, tol: float, mask: int = 0xFFFF, summed: bool = False,
                  skip: int = 0, count: int = -1) -> Tuple[bool, float, int]:
    """Returns (pass, largest error, line of the largest error); file_a drives
    the line loop; paths or lists of lines are accepted."""
    def lines(src):
        if isinstance(src, (list, tuple)):
            return list(src)
        with open(src) as fh:
            return fh.read().splitlines()

    la, lb = lines(file_a), lines(file_b)
    ntok = bin(mask).count("1")
    ok, worst, worst_line = True, 0.0, -1
    line = skip
    for k in range(skip, len(la)):
        ta = la[k].split(" ")
        tb = lb[k].split(" ") if k < len(lb) else []
        sa = sb = 0.0
        n = 0
        for t, item in enumerate(ta):
            if not (mask >> t) & 1:
                continue
            a, b = float(item), float(tb[t] if t < len(tb) else "nan")
            res = None
            if summed and n < ntok:
                sa, sb, n = sa + a, sb + b, n + 1
                if n == ntok:
                    res = _relative_or_absolute(sa, sb, tol)
            else:
                res = _relative_or_absolute(a, b, tol)
            if res is not None:
                ok = ok and res[0]
                if res[1] > worst:
                    worst, worst_line = res[1], line
        line += 1
        if count > 0 and line - skip >= count:
            break
    return ok, worst, worst_line


def two_stream_em_rule(gold, ours, tol: float = 0.10):
    """The 2stream-em regression rule: E (token 2) and B (token 3) separately,
    lines 3581..4880, 10% relative."""
    return (compare_files(gold, ours, tol, 0b100, True, 3581, 1300),
            compare_files(gold, ours, tol, 0b1000, True, 3581, 1300))
