"""The reference's output files and printed blocks (list-directed records,
the fort.7 / err_table.dat order-table flow), produced from oracle runs on
the CPU."""
import math

import numpy as np

from sweeping_fd_weno_gb300 import abi, problems
from sweeping_fd_weno_gb300.output import e13_5, fortran_real, list_record, write_output


def test_list_directed_items():
    assert list_record(1.0) == "   1.0000000000000000     "
    assert list_record(0.5) == "  0.50000000000000000     "
    assert list_record(1e-2) == "   1.0000000000000000E-002"
    assert list_record(-1.0) == "  -1.0000000000000000     "
    assert list_record(1e16) == "   10000000000000000.     "
    assert list_record(1e17) == "   1.0000000000000000E+017"
    assert list_record("total sweep = ", 5) == " total sweep =            5"
    assert list_record("L1 = ", " Linfinity =") == " L1 =  Linfinity ="
    assert list_record("zone i=", 104, ", j=", 88) == " zone i=         104 , j=          88"
    assert len(fortran_real(math.pi)) == 25
    assert e13_5(1.0) + e13_5(-3.0) == "  0.10000E+01 -0.30000E+01"


class OracleRun:
    """The attributes `write_output` reads, from an oracle run."""

    def __init__(self, oracle_mod, cfg, steps=0):
        self.cfg = cfg
        self.o = oracle_mod.Oracle(cfg)
        self.o.init_problem()
        if steps:
            for _ in range(steps):
                self.o.step()
        else:
            self.o.run()
        self.time = self.o.time

    def state(self):
        return self.o.state()

    def stats(self):
        return self.o.stats()

    def _dx(self):
        return self.o.dx

    def _dy(self):
        return self.o.dy


def test_vortex_order_table_flow(oracle_mod, tmp_path):
    """Two resolutions through fort.7 / err_table.dat (the Table-1 flow,
    ex3_vortex_accuracy_2d/main.f90:745-777): the second row carries the
    fifth-order convergence rate."""
    r90 = OracleRun(oracle_mod, problems.workload("vortex90"))
    write_output(r90, tmp_path, new_table=True, ierror=0)
    r180 = OracleRun(oracle_mod, problems.workload("vortex180"))
    t2 = write_output(r180, tmp_path, new_table=False, ierror=1)
    rows = (tmp_path / "err_table.dat").read_text().splitlines()
    assert len(rows) == 2
    n0, e10, o10, ei0, oi0 = rows[0].split()
    n1, e11, o11, ei1, oi1 = rows[1].split()
    assert (int(n0), int(n1)) == (90, 180) and float(o10) == 0.0
    assert 4.0 < float(o11) < 6.5, o11
    f7 = (tmp_path / "fort.7").read_text().rstrip("\n")
    assert len(f7) == 26 and f7[2:4] == "0." and float(f7[:13]) == float(e13_5(float(e11)))
    assert " L1 =  Linfinity =" in t2 and " total sweep = " in t2
    den = (tmp_path / "den.dat").read_text().splitlines()
    assert len(den) == 180 * 180 and len(den[0].split()) == 5
    for name in ("pre.dat", "m1.dat", "m2.dat", "den2.dat", "pre2.dat"):
        assert len((tmp_path / name).read_text().splitlines()) == 180 * 180


def test_point_energy_jet_and_shock_files(oracle_mod, tmp_path):
    s = OracleRun(oracle_mod, problems.make_config(abi.SEDOV_2D, nx=16, ny=12), steps=2)
    write_output(s, tmp_path / "ex4")
    den = (tmp_path / "ex4" / "den.dat").read_text().splitlines()
    assert den[0] == ' VARIABLES = "X", "Y", "DENSITY"'
    assert den[1] == list_record("zone i=", 16, ", j=", 12)
    assert len(den) == 2 + 16 * 12
    j = OracleRun(oracle_mod, problems.make_config(abi.JET_2D, nx=16, ny=8), steps=1)
    write_output(j, tmp_path / "ex5")
    den = (tmp_path / "ex5" / "den.dat").read_text().splitlines()
    assert den[1] == list_record("zone i=", 16, ", j=", 16) and len(den) == 2 + 2 * 16 * 8
    # mirrored lower half: its first row is the top row of the grid, y shifted by -0.25
    first = [float(v) for v in den[2].split()]
    assert abs(first[1] - (0.25 / 8 * 0.5 - 0.25)) < 1e-15
    sh = OracleRun(oracle_mod, problems.workload("shock12"), steps=1)
    write_output(sh, tmp_path / "ex6")
    den = (tmp_path / "ex6" / "den.dat").read_text().splitlines()
    assert den[0] == list_record("zone i=", 12 * 13, ", j=", 12 * 11)
    vals = np.array([[float(v) for v in r.split()] for r in den[1:]])
    assert (vals[0, 2] == 0.0) and (vals[:, 2] > 0).any()  # the step region is written as 0


def test_detonation_files(oracle_mod, tmp_path):
    """ex7's output: den.dat, pre.dat (pressure with the q*Y term) and rate.dat
    (Y = rho*Y/rho) over 5*total x 5*total cells, the step region written as
    100, 300 and 20."""
    d = OracleRun(oracle_mod, problems.make_config(abi.DETONATION, total=8, cut_x=2, cut_y=2),
                  steps=2)
    text = write_output(d, tmp_path / "ex7")
    for name, fill in (("den.dat", 100.0), ("pre.dat", 300.0), ("rate.dat", 20.0)):
        rows = (tmp_path / "ex7" / name).read_text().splitlines()
        assert rows[0] == list_record("zone i=", 40, ", j=", 40)
        vals = np.array([[float(v) for v in r.split()] for r in rows[1:]])
        assert vals.shape == (40 * 40, 3)
        assert vals[0, 2] == fill and (vals[:, 2] != fill).any()
    assert " total sweep = " in text
