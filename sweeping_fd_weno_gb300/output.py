"""The reference's `output` routines: .dat files, the printed statistics block,
and the L1/Linf order-table flow (fort.7 and err_table.dat) of the accuracy
study.

Every example writes its own files (ex2_sedov_1d/main.f90:441-513,
ex3_vortex_accuracy_2d/main.f90:720-841, ex4_sedov_2d/main.f90:1193-1354,
ex5_mach2000_jet/main.f90 `output`, ex6_shock_diffraction/main.f90:1154-1264)
with Fortran list-directed WRITE (*) records.  Records are formatted here by
gfortran's list-directed rules for default integers and REAL(8): a blank
before every item except a character item that follows a character item,
integers right-justified in 11 columns, reals in 25 columns with 17
significant digits, fixed form for 0.1 <= |x| < 1e17 (followed by the 5
blanks that stand for the exponent) and exponent form with a 3-digit exponent
otherwise.  fort.7 uses the explicit format (6e13.5).  No Fortran compiler
was available to compare these files byte for byte with the reference's.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

from . import abi

_REAL_W = 25   # list-directed width of a REAL(8)
_INT_W = 11    # list-directed width of a default INTEGER
_SIG = 17      # significant digits of a REAL(8)


def fortran_real(v: float) -> str:
    """One list-directed REAL(8) item (25 columns)."""
    v = float(v)
    if math.isnan(v):
        return "NaN".rjust(_REAL_W)
    if math.isinf(v):
        return ("-Infinity" if v < 0 else "Infinity").rjust(_REAL_W)
    a = abs(v)
    if a == 0.0:
        z = ("-" if math.copysign(1.0, v) < 0 else "") + "0." + "0" * (_SIG - 1)
        return z.rjust(_REAL_W - 5) + " " * 5
    # round to 17 significant digits first: the form follows the rounded value
    m, e = f"{a:.{_SIG - 1}e}".split("e")
    ex = int(e)
    if -1 <= ex < _SIG:
        k = ex + 1                       # integer digits (0 for 0.1 <= a < 1)
        s = f"{a:.{_SIG - k}f}"
        if k == 0 and s.startswith("1."):  # rounded up to 1.0: one digit more
            s = f"{a:.{_SIG - 1}f}"
        if k == _SIG:
            s = s + "."
        if v < 0:
            s = "-" + s
        return s.rjust(_REAL_W - 5) + " " * 5
    s = f"{m}E{'+' if ex >= 0 else '-'}{abs(ex):03d}"
    if v < 0:
        s = "-" + s
    return s.rjust(_REAL_W)


def fortran_int(v: int) -> str:
    return str(int(v)).rjust(_INT_W)


def list_record(*items) -> str:
    """One list-directed output record (without the newline)."""
    out = []
    prev_char = False
    for k, it in enumerate(items):
        is_char = isinstance(it, str)
        if k == 0 or not (is_char and prev_char):
            out.append(" ")
        if is_char:
            out.append(it)
        elif isinstance(it, (int, np.integer)) and not isinstance(it, bool):
            out.append(fortran_int(it))
        else:
            out.append(fortran_real(it))
        prev_char = is_char
    return "".join(out)


def e13_5(v: float) -> str:
    """Fortran E13.5: 0.ddddd E+ee, right-justified in 13 columns."""
    v = float(v)
    if v == 0.0:
        return "0.00000E+00".rjust(13)
    m, e = f"{abs(v):.4e}".split("e")
    digits = m.replace(".", "")
    ex = int(e) + 1
    s = f"0.{digits}E{'+' if ex >= 0 else '-'}{abs(ex):02d}"
    return ("-" + s if v < 0 else s).rjust(13)


def stats_block(st: dict) -> str:
    """The statistics lines printed at the end of `output`
    (ex3_vortex_accuracy_2d/main.f90:815-840)."""
    n = st["sweep_count"]
    avg = (lambda t: float(t) / float(n)) if n else (lambda t: float("nan"))
    lines = [
        list_record("total sweep = ", st["total_sweep"]),
        list_record("avg sweep = ", avg(st["total_sweep"])),
        list_record("max sweep = ", st["max_sweep"]),
        list_record("total negative pairs = ", st["total_neg"]),
        list_record("avg negative pairs = ", avg(st["total_neg"])),
        list_record("max negative pairs = ", st["max_neg"]),
        list_record("total positive neighbors = ", st["total_pos"]),
        list_record("avg positive neighbors = ", avg(st["total_pos"])),
        list_record("max positive neighbors = ", st["max_pos"]),
        list_record("# of limiter", st["den_count"], st["pre_count"]),
    ]
    return "\n".join(lines) + "\n"


def vortex_exact(x: float, y: float, t: float, gamma: float = 1.4):
    """`exact` of ex3_vortex_accuracy_2d/main.f90:698-718, same operation order."""
    g1 = gamma - 1.0
    pi = 3.14159265358979323846264338327950
    r = math.sqrt((x - 5. - t) * (x - 5. - t) + (y - 5. - t) * (y - 5. - t))
    mag = 10.0828
    e1 = math.pow(1 - g1 * (mag * mag) / 8. / gamma / (pi * pi) * math.exp(1. - r * r), 1. / g1)
    e2 = e1 * (1. - mag / 2. / pi * math.exp((1. - r * r) / 2.) * (y - 5.))
    e3 = e1 * (1. + mag / 2. / pi * math.exp((1. - r * r) / 2.) * (x - 5.))
    e4 = math.pow(e1, gamma) / g1 + 0.5 * (e2 * e2) / e1 + 0.5 * (e3 * e3) / e1
    return e1, e2, e3, e4


def vortex_errors(u, t: float, gamma: float = 1.4):
    """L1 (mean over the interior) and Linf density errors of a vortex state
    u(-2:ny+3, -2:nx+3, 4) against `exact` at time t, as
    ex3_vortex_accuracy_2d/main.f90:725-745 computes them (vectorised; the
    exact density follows vortex_exact's formula)."""
    import numpy as np
    ny, nx = u.shape[0] - 6, u.shape[1] - 6
    dx, dy = 10. / nx, 10. / ny
    x = np.arange(1, nx + 1) * dx - dx / 2.
    y = np.arange(1, ny + 1) * dy - dy / 2.
    X, Y = np.meshgrid(x, y)
    g1 = gamma - 1.0
    pi = 3.14159265358979323846264338327950
    r2 = (X - 5. - t) * (X - 5. - t) + (Y - 5. - t) * (Y - 5. - t)
    mag = 10.0828
    e1 = np.power(1 - g1 * (mag * mag) / 8. / gamma / (pi * pi) * np.exp(1. - r2), 1. / g1)
    d = np.abs(e1 - u[3:ny + 3, 3:nx + 3, 0])
    return float(d.sum() / nx / ny), float(d.max())


def _read_fort7(path: Path):
    """read (7, '(6e13.5)') er1old, eriold"""
    txt = path.read_text() if path.exists() else ""
    line = (txt.splitlines() or [""])[0]
    vals = [line[k:k + 13] for k in range(0, 26, 13)]
    try:
        return tuple(float(v.replace("D", "E")) for v in vals)
    except ValueError:
        raise ValueError(f"{path}: expected two E13.5 fields, got {line!r}")


def _order_table(out: Path, n: int, er1: float, eri: float, ierror: int,
                 new_table: bool | None):
    """fort.7 / err_table.dat flow: the previous resolution's errors give the
    orders, the current ones replace them (ex3_vortex_accuracy_2d/main.f90:745-777)."""
    er1old, eriold = 1., 1.
    if ierror == 1:
        er1old, eriold = _read_fort7(out / "fort.7")
    o1 = math.log(er1old / er1) / math.log(2.0)
    oi = math.log(eriold / eri) / math.log(2.0)
    text = (list_record("L1 = ", " Linfinity =") + "\n" + list_record(er1, eri) + "\n" +
            list_record("L1order=", " Liorder=") + "\n" + list_record(o1, oi) + "\n")
    if new_table is not None:
        if new_table:
            o1, oi = 0.0, 0.0
        mode = "w" if new_table else "a"
        with open(out / "err_table.dat", mode) as f:
            f.write(list_record(int(n), er1, o1, eri, oi) + "\n")
    (out / "fort.7").write_text(e13_5(er1) + e13_5(eri) + "\n")
    return text


def _cols(path: Path, rows, header=()):
    with open(path, "w") as f:
        for h in header:
            f.write(h + "\n")
        for r in rows:
            f.write(list_record(*r) + "\n")


def write_output(solver, out_dir: str | Path = ".", new_table: bool | None = False,
                 ierror: int | None = None) -> str:
    """Write the example's .dat files into out_dir and return the text its
    `output` prints (errors and orders where the example computes them, then
    the statistics block).  For the vortex, new_table / ierror are the
    PARAMETERs of ex3_vortex_accuracy_2d/main.f90:5,9 (None: no err_table.dat)."""
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    cfg = solver.cfg
    p = cfg.problem
    u = solver.state()
    g1 = cfg.gamma - 1.0
    text = ""
    if p == abi.SEDOV_1D:
        # ex2_sedov_1d/main.f90:441-486
        n = cfg.nx
        dx = (2. - (-2.)) / n
        x = [-2. + i * dx - dx / 2. for i in range(1, n + 1)]
        pi = 3.14159265358979323846264338327950
        er1, eri = 0., 0.
        for i in range(1, n + 1):
            ex1 = 1. + 0.99999999 * math.sin(2 * pi * (x[i - 1] - solver.time))
            d = abs(ex1 - u[0, i + 2, 0])
            er1 = er1 + d
            eri = max(eri, d)
        er1 = er1 / n
        text += _order_table(out, n, er1, eri, 0 if ierror is None else ierror, None)
        r = u[0, 3:n + 3, :]
        _cols(out / "den.dat", ((x[i], r[i, 0]) for i in range(n)))
        _cols(out / "pre.dat", ((x[i], g1 * (r[i, 2] - 0.5 * (r[i, 1] * r[i, 1]) / r[i, 0]))
                               for i in range(n)))
        _cols(out / "vel.dat", ((x[i], r[i, 1] / r[i, 0]) for i in range(n)))
    elif p == abi.VORTEX_2D:
        # ex3_vortex_accuracy_2d/main.f90:720-813
        nx, ny = cfg.nx, cfg.ny
        dx, dy = 10. / nx, 10. / ny
        x = [0. + i * dx - dx / 2. for i in range(1, nx + 1)]
        y = [0. + j * dy - dy / 2. for j in range(1, ny + 1)]
        t = solver.time
        ex = [[vortex_exact(x[i], y[j], t, cfg.gamma)[0] for j in range(ny)] for i in range(nx)]
        er1, eri = 0., 0.
        for i in range(nx):
            for j in range(ny):
                d = abs(ex[i][j] - u[j + 3, i + 3, 0])
                er1 = er1 + d
                eri = max(eri, d)
        er1 = er1 / nx / ny
        text += _order_table(out, nx, er1, eri, 1 if ierror is None else ierror, new_table)
        pre = lambda v: g1 * (v[3] - 0.5 * (v[1] * v[1]) / v[0] - 0.5 * (v[2] * v[2]) / v[0])
        cells = [(i, j) for j in range(ny) for i in range(nx)]
        _cols(out / "den.dat", ((x[i], y[j], u[j + 3, i + 3, 0], ex[i][j],
                                 abs(ex[i][j] - u[j + 3, i + 3, 0])) for i, j in cells))
        _cols(out / "pre.dat", ((x[i], y[j], pre(u[j + 3, i + 3])) for i, j in cells))
        _cols(out / "m1.dat", ((x[i], y[j], u[j + 3, i + 3, 1]) for i, j in cells))
        _cols(out / "m2.dat", ((x[i], y[j], u[j + 3, i + 3, 2]) for i, j in cells))
        _cols(out / "den2.dat", ((y[j], u[j + 3, i + 3, 0]) for i, j in cells))
        _cols(out / "pre2.dat", ((y[j], pre(u[j + 3, i + 3])) for i, j in cells))
    elif p in (abi.SEDOV_2D, abi.JET_2D, abi.SHOCK_DIFFRACTION):
        nx, ny = cfg.nx, cfg.ny
        dx, dy = solver._dx(), solver._dy()
        v = u[3:ny + 3, 3:nx + 3, :]
        pres = g1 * (v[..., 3] - 0.5 * (v[..., 1] * v[..., 1]) / v[..., 0]
                     - 0.5 * (v[..., 2] * v[..., 2]) / v[..., 0])
        xs = [dx * (i - 0.5) for i in range(1, nx + 1)]
        ys = [dy * (j - 0.5) for j in range(1, ny + 1)]
        cells = [(i, j) for j in range(ny) for i in range(nx)]
        if p == abi.SEDOV_2D:
            # ex4_sedov_2d/main.f90:1270-1320
            zone = list_record("zone i=", int(nx), ", j=", int(ny))
            var = list_record('VARIABLES = "X", "Y", "DENSITY"')
            _cols(out / "den.dat", ((xs[i], ys[j], v[j, i, 0]) for i, j in cells), (var, zone))
            _cols(out / "pre.dat", ((xs[i], ys[j], pres[j, i]) for i, j in cells), (zone,))
            _cols(out / "m1.dat", ((xs[i], ys[j], v[j, i, 1]) for i, j in cells), (zone,))
            _cols(out / "m2.dat", ((xs[i], ys[j], v[j, i, 2]) for i, j in cells), (zone,))
        elif p == abi.JET_2D:
            # ex5_mach2000_jet `output`: the lower half mirrored, then the upper half;
            # log |rho|, log |p|, log |p/rho| (m1.dat)
            zone = list_record("zone i=", int(nx), ", j=", int(2 * ny))
            var = list_record('VARIABLES = "X", "Y", "DENSITY"')
            low = [(i, j) for j in range(ny) for i in range(nx)]

            def rows(kind):
                for i, j in low:          # j -> row ny - j (mirrored), y shifted by -0.25
                    jj = ny - 1 - j
                    yield xs[i], ys[j] - 0.25, kind(jj, i)
                for i, j in low:
                    yield xs[i], ys[j], kind(j, i)
            _cols(out / "den.dat", rows(lambda j, i: math.log(abs(v[j, i, 0]))), (var, zone))
            _cols(out / "pre.dat", rows(lambda j, i: math.log(abs(pres[j, i]))), (zone,))
            _cols(out / "m1.dat", rows(lambda j, i: math.log(abs(pres[j, i] / v[j, i, 0]))),
                  (zone,))
        else:
            # ex6_shock_diffraction/main.f90:1195-1220: the step region written as 0
            total = cfg.total
            zone = list_record("zone i=", int(total * 13), ", j=", int(total * 11))

            def val(arr, i, j):
                return 0. if (i + 1 < total and j + 1 < 6 * total) else arr
            _cols(out / "den.dat", ((xs[i], ys[j], val(v[j, i, 0], i, j)) for i, j in cells),
                  (zone,))
            _cols(out / "pre.dat", ((xs[i], ys[j], val(pres[j, i], i, j)) for i, j in cells),
                  (zone,))
    elif p == abi.DETONATION:
        # ex7_detonation/main.f90:1264-1394: density, pressure (with the q*Y
        # term) and the mass fraction Y over 5*total x 5*total cells, the step
        # region written as 100, 300 and 20
        total = cfg.total
        n = 5 * total
        dx, dy = solver._dx(), solver._dy()
        q = 50.
        zone = list_record("zone i=", n, ", j=", n)
        den, pre, rate = [], [], []
        for j in range(n):
            for i in range(n):
                lrho, lm, ln, le, ly = (float(c) for c in u[j + 3, i + 3, :5])
                pres = g1 * (le - 0.5 * (lm * lm) / lrho - 0.5 * (ln * ln) / lrho - q * ly)
                yr = ly / lrho
                if i + 1 <= total and j + 1 < 2 * total:
                    lrho, pres, yr = 100., 300., 20.
                xy = (dx * (i + 1 - 0.5), dy * (j + 1 - 0.5))
                den.append(xy + (lrho,))
                pre.append(xy + (pres,))
                rate.append(xy + (yr,))
        _cols(out / "den.dat", den, (zone,))
        _cols(out / "pre.dat", pre, (zone,))
        _cols(out / "rate.dat", rate, (zone,))
    text += stats_block(solver.stats())
    return text
