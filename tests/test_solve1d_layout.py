"""The persistent 1D solve's index arithmetic, on the CPU: for every block of
every shape the launcher accepts (6..62 cells per block, at most 256 blocks),
the kernel's own layout function (solve1d_layout, through the probe library)
keeps each access of the kernel in bounds and each halo cell in a direct
neighbour's range -- the invariants the kernel's shared-memory arrays and
its left/right ready flags rely on.  Cells sit at offsets 0..nx+5 (cell i of
ex2_sedov_1d/main.f90 at i + 2, three ghosts a side); the interface-flux
cells are the reference's m = 0..nx+1 (:88-157), offsets 2..nx+3."""
import ctypes as C

from sweeping_fd_weno_gb300 import abi

MIN_CELLS, MAX_CELLS, MAX_BLOCK, MAX_GRID = 6, 62, 512, 4 * 64

NX = list(range(1, 41)) + [100, 154, 155, 159, 160, 200, 400, 799, 800, 801, 802, 803, 804,
                           805, 906, 907, 912, 1000, 1500, 2000, 3000, 5000, 9000, 15000]


def _layout(probe, nx, cells, b):
    out = (C.c_int32 * 10)()
    assert probe.swfd_probe_solve1d_layout(nx, cells, b, out) == abi.OK
    return dict(zip(("a0", "a1", "nown", "f0", "f1", "nf", "s0", "ns", "nhl", "nhr"), out))


def test_layout_rejects_blocks_past_the_cells(swfd):
    probe = abi.load_probe()
    out = (C.c_int32 * 10)()
    assert probe.swfd_probe_solve1d_layout(10, 6, 3, out) == abi.ERR_INVALID  # 16 cells: 0..2
    assert probe.swfd_probe_solve1d_layout(10, 6, 2, out) == abi.OK
    assert probe.swfd_probe_solve1d_layout(0, 6, 0, out) == abi.ERR_INVALID


def test_every_shape_stays_in_bounds(swfd):
    probe = abi.load_probe()
    shapes = 0
    for nx in NX:
        LI = nx + 6
        for cells in range(MIN_CELLS, MAX_CELLS + 1):
            grid = -(-LI // cells)
            block = min(MAX_BLOCK, max(128, (16 * (cells + 2) + 31) // 32 * 32))
            if grid > MAX_GRID or 4 * cells > block:
                continue  # the launcher declines these shapes
            shapes += 1
            SW, FW = cells + 6, cells + 2
            lay = [_layout(probe, nx, cells, b) for b in range(grid)]
            owner = {}
            for b, L in enumerate(lay):
                for q in range(L["a0"], L["a1"]):
                    assert q not in owner
                    owner[q] = b
            assert sorted(owner) == list(range(LI)), (nx, cells)
            for b, L in enumerate(lay):
                ctx = (nx, cells, b, L)
                a0, a1, f0, f1, nf, s0, ns = (L[k] for k in ("a0", "a1", "f0", "f1", "nf", "s0",
                                                             "ns"))
                assert L["nown"] == a1 - a0 >= 1, ctx
                # shared arrays: split cells (state, fflux, split) SW wide,
                # flux cells (fluxes, eigenvectors) FW wide
                assert 0 <= s0 and s0 + ns <= LI, ctx
                assert ns <= SW and 0 <= nf <= FW, ctx
                assert s0 <= a0 and a1 <= s0 + ns, ctx
                assert s0 == f0 - 2 and s0 + ns - 1 == f1 + 2, ctx
                assert 2 <= f0 and f1 <= nx + 3, ctx
                # halo: at most three cells a side, each owned by the block
                # next to this one (the two ready flags a block waits for)
                assert 0 <= L["nhl"] <= 3 and 0 <= L["nhr"] <= 3, ctx
                assert L["nhl"] == a0 - s0 and a1 + L["nhr"] == s0 + ns, ctx
                for q in range(s0, a0):
                    assert owner[q] == b - 1, ctx
                for q in range(a1, a1 + L["nhr"]):
                    assert owner[q] == b + 1, ctx
                # (with no flux cell, nf = 0, f0 is still read: the last
                # owned cell of the block before)
                if f0 < a0:
                    assert owner[f0] == b - 1, ctx
                if f1 >= a1:
                    assert owner[f1] == b + 1, ctx
                # the halo copy on the 64 threads of warps 2 and 3: six values
                # a halo cell from the first, fifteen eigenvector values a
                # flux cell next to the range from the last
                assert 6 * (L["nhl"] + L["nhr"]) <= 64 and 2 * 15 <= 64, ctx
                # the RK stage reads the fluxes k - 1 .. k + 1 of an interior cell
                for q in range(a0, a1):
                    if 1 <= q - 2 <= nx:
                        k = q - f0
                        assert 1 <= k and k + 1 <= nf - 1, ctx
                # threads: split (one component per group of warps), sixteen
                # lanes per flux cell in turns, four per owned cell in the RK stage
                assert ns <= block and 4 * L["nown"] <= block, ctx
    assert shapes > 1000
