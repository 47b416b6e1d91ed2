"""Text writers that reproduce BraWl's output files byte-for-byte.

* energy trajectory   -- energy_trajectory_writer, format (I13,x,f20.10,x)
                         (src/metropolis_output.f90:34-53)
* ASRO trajectory     -- asro_trajectory_writer, (I13,x) then (f8.5,x) per
                         value, i fastest (src/metropolis_output.f90:66-98)
* energy diagnostics  -- diagnostics_writer,
                         (F8.1,2X,F24.15,2X,F24.15,2X,F6.4)
                         (src/metropolis_output.f90:113-135)
* NS energies         -- list-directed write of (i_iter, ener_limit)
                         (src/nested_sampling.f90:80-84, 121)

Header lines come from list-directed writes of a string, which gfortran
prefixes with one blank.  A trailing X edit descriptor at the end of a record
writes nothing.
"""
from __future__ import annotations

import numpy as np


def energy_trajectory_header() -> str:
    return " # step_number E\n"


def energy_trajectory_line(step: int, energy: float) -> str:
    return "%13d %20.10f\n" % (step, energy)


def asro_trajectory_header() -> str:
    return " # step_number ASRO\n"


def asro_trajectory_line(step: int, asro: np.ndarray) -> str:
    """asro shaped (wc_range, ns, ns): the C view of asro(i, j, k), so a
    row-major ravel visits i fastest, then j, then k, as the reference."""
    vals = np.asarray(asro, dtype=np.float64).ravel()
    return "%13d " % step + "".join("%8.5f " % v for v in vals) + "\n"


def diagnostics_lines(temps, energies, C, acceptance) -> list[str]:
    out = [" # T E C acceptance_rate\n"]
    for t, e, c, a in zip(temps, energies, C, acceptance):
        out.append("%8.1f  %24.15f  %24.15f  %6.4f\n" % (t, e, c, a))
    return out


def _g_real8(x: float) -> str:
    """gfortran list-directed REAL(8): a G25.17-style field (17 significant
    digits, 4 trailing blanks in F form) after one separating blank."""
    ax = abs(x)
    if ax != 0.0 and (ax < 0.1 or ax >= 1e16):
        mant = "%.16E" % x
        m, e = mant.split("E")
        s = "%sE%+04d" % (m, int(e))
        return " " + s.rjust(25)
    digits_before = 1 if ax < 1.0 else len(str(int(ax)))
    decimals = max(17 - digits_before, 0)
    if ax < 1.0:
        decimals = 17
    s = ("%." + str(decimals) + "f") % x
    return " " + s.rjust(20) + "     "


def ns_energies_header(n_walkers: int, n_at: int) -> str:
    return "%12d%12d%12d False%12d\n" % (n_walkers, 1, 0, n_at)


def ns_energies_line(i_iter: int, limit: float) -> str:
    return "%12d%s\n" % (i_iter, _g_real8(limit))
