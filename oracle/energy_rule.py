"""Energy-history comparison rule of the reference's regression test.

Restates tests/energy_comparison/compare_energies.h (compare_error at :69-106,
compare_energies at :135-362) as used by tests/energy_comparison/2stream-em.cxx
(:45-70): skip N lines of both files, then for each of the next M lines sum the
masked whitespace-separated tokens (bit k of the mask selects token k, token 0
being the step) and compare the sums with a relative tolerance; when the
smaller value is below 10 double epsilons an absolute test at 2 epsilons is
used instead.  Test infrastructure only.
"""
from __future__ import annotations

import sys
from typing import Iterable, List, Sequence, Tuple

_EPS = sys.float_info.epsilon


def compare_error(a: float, b: float, rel_tol: float) -> Tuple[bool, float]:
    """compare_energies.h:69-106: relative error |a-b|/min(a,b), absolute near 0."""
    if abs(min(a, b)) < 10 * _EPS:
        err = abs(a - b)
        return err < 2 * _EPS, err
    err = abs(a - b) / min(a, b)
    return err < rel_tol, err


def _lines(src) -> List[str]:
    if isinstance(src, (list, tuple)):
        return list(src)
    with open(src) as fh:
        return fh.read().splitlines()


def compare_energies(file_a, file_b, rel_tol: float, field_mask: int = 0xFFFF,
                     sum_fields: bool = False, skip: int = 0, lines_to_read: int = -1):
    """Returns (match, max_err, max_err_line, errors).

    file_a drives the loop, as in the reference (while getline(f1, ...)).
    file_a / file_b may be paths or lists of lines.
    """
    la, lb = _lines(file_a), _lines(file_b)
    agg_total = bin(field_mask).count("1")
    match = True
    max_err, max_line = 0.0, -1
    errs: List[float] = []
    counter = skip
    for k in range(skip, len(la)):
        ta = la[k].split(" ")
        tb = lb[k].split(" ") if k < len(lb) else []
        sum_a = sum_b = 0.0
        agg = 0
        for t, item_a in enumerate(ta):
            item_b = tb[t] if t < len(tb) else ""
            if not (field_mask >> t) & 1:
                continue
            a, b = float(item_a), float(item_b)
            result = None
            if sum_fields and agg < agg_total:
                sum_a += a
                sum_b += b
                agg += 1
                if agg == agg_total:
                    result = compare_error(sum_a, sum_b, rel_tol)
            else:
                result = compare_error(a, b, rel_tol)
            if result is not None:
                ok, err = result
                match = match and ok
                if err > max_err:
                    max_err, max_line = err, counter
                errs.append(err)
        counter += 1
        if lines_to_read > 0 and counter - skip >= lines_to_read:
            break
    return match, max_err, max_line, errs


def two_stream_em_check(gold, ours, rel_tol: float = 0.10):
    """The 2stream-em finalizer (2stream-em.cxx:45-70): E (token 2) and B
    (token 3) separately, skip 3581 lines, read 1300, 10% relative."""
    e = compare_energies(gold, ours, rel_tol, 0b100, True, 3581, 1300)
    b = compare_energies(gold, ours, rel_tol, 0b1000, True, 3581, 1300)
    return e, b


def format_energy_line(step: int, time: float, e: float, b: float) -> str:
    """dump_energies line (src/fields.h:752-756): `step time E B` written by a
    std::ostream at its default precision of 6 significant digits."""
    return f"{step} {_g6(time)} {_g6(e)} {_g6(b)}"


def _g6(v: float) -> str:
    s = f"{v:.6g}"
    if "e" in s:  # ostream prints a two-digit exponent at least, like %g
        mant, exp = s.split("e")
        sign = exp[0]
        digits = exp[1:].lstrip("0") or "0"
        s = f"{mant}e{sign}{digits.zfill(2)}"
    return s


def format_history(rows: Iterable[Sequence[float]], dt: float) -> List[str]:
    return [format_energy_line(i + 1, (i + 1) * dt, r[0], r[1]) for i, r in enumerate(rows)]
