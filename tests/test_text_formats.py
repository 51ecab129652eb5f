"""The reference's text outputs (tc_format_g, tc_format_stats_line,
tc_format_vis_line of tracer_gpu.h; host-only calls through the C ABI).

  - every g20.8 field of the shipped stats.dat, viscosity_smoother.dat and
    equalize.dat re-formats from its value to the same characters;
  - every shipped stats.dat and viscosity_smoother.dat row comes back byte
    for byte from its values (the comp = 0, tracer = 1 branches of
    basics.f90:283-322);
  - the other branches have the reference's field counts and widths, and the
    Gw.dEe form of the snapshots follows the same rules.
"""
import pytest

from tracer_code_gb300 import build as tcbuild

STATS_COLS = ["time", "Tavg", "vrms", "Nu", "Nu_bot", "RaT_avg", "mobility", "strain_max", "q1", "q2", "q3", "q4"]


@pytest.fixture(scope="module")
def tio():
    tcbuild.build()
    from tracer_code_gb300 import textio
    return textio


def fields(line, widths):
    out, pos = [], 0
    for w in widths:
        out.append(line[pos:pos + w])
        pos += w
    assert pos == len(line)
    return out


SPECS = {"stats.dat": [20] * 12 + [6] * 3, "viscosity_smoother.dat": [20, 5, 20, 5], "equalize.dat": [20] + [10] * 6}


@pytest.mark.parametrize("name", sorted(SPECS))
def test_every_shipped_real_field_reformats(tio, golden, name):
    n = 0
    for line in golden["text_lines"][name]:
        for f, w in zip(fields(line, SPECS[name]), SPECS[name]):
            if w == 20:
                assert tio.format_g(float(f), 20, 8) == f
                n += 1
            else:
                assert f == f"{int(f):>{w}d}"
    assert n >= 17


def test_shipped_stats_rows_come_back_byte_for_byte(tio, golden):
    lines = golden["text_lines"]["stats.dat"]
    assert len(lines) == golden["stats_rows"]
    for line in lines:
        f = fields(line, SPECS["stats.dat"])
        row = {c: float(v) for c, v in zip(STATS_COLS, f)}
        row.update(empty_cells=int(f[12]), tracer_min=int(f[13]), tracer_max=int(f[14]))
        assert tio.stats_line(row, comp=0, tracer=1, ntype=0, RaT=golden["inputs"]["RaT"]) == line


def test_shipped_viscosity_rows_come_back_byte_for_byte(tio, golden):
    for line in golden["text_lines"]["viscosity_smoother.dat"]:
        f = fields(line, SPECS["viscosity_smoother.dat"])
        row = {"time": float(f[0]), "n_eta": int(f[1]), "eig_fine": float(f[2]), "n_temp": int(f[3])}
        assert tio.vis_line(row, comp=0, ntype=0, RaT=golden["inputs"]["RaT"]) == line


def test_branch_layouts(tio):
    row = {c: 0.5 + i for i, c in enumerate(STATS_COLS)}
    row.update(empty_cells=3, tracer_min=7, tracer_max=41, Cavg=[0.1, 0.2], ent=[0.3, 0.4], n_eta=2, n_temp=1,
               n_comp=[5, 6], eig_fine=4.25)
    assert len(tio.stats_line(row, 0, 0, 0, 1e5)) == 12 * 20
    assert len(tio.stats_line(row, 0, 1, 0, 1e5)) == 12 * 20 + 3 * 6
    s = tio.stats_line(row, 1, 0, 2, 1e5)
    assert len(s) == 12 * 20 + 3 * 6 + 4 * 20
    assert s[240:258] == "     3     7    41"
    assert s[258:].split() == ["0.10000000", "0.20000000", "0.30000000", "0.40000000"]
    assert len(tio.stats_line(row, 0, 0, 0, 0.0)) == 4 * 20
    assert len(tio.stats_line(row, 1, 0, 1, 0.0)) == 4 * 20 + 3 * 6 + 2 * 20
    assert tio.vis_line(row, 1, 2, 1e5) == tio.format_g(row["time"], 20, 8) + "    2" + \
        tio.format_g(4.25, 20, 8) + "    1    5    6"
    assert tio.vis_line(row, 1, 2, 0.0).endswith("    2" + tio.format_g(4.25, 20, 8) + "    5    6")
    assert tio.vis_line(row, 0, 0, 0.0) == ""


@pytest.mark.parametrize("x,w,d,e,want", [
    (0.0, 20, 8, 0, "       0.0000000    "),
    (-0.0, 14, 5, 3, "  -0.0000     "),
    (1.0, 14, 5, 3, "   1.0000     "),
    (0.1, 14, 5, 3, "  0.10000     "),
    (99999.4, 14, 5, 3, "   99999.     "),        # F9.0 keeps the decimal point
    (99999.5, 14, 5, 3, "  0.10000E+006"),        # rounds to 6 digits before the point: E form
    (0.0999996, 14, 5, 3, "  0.10000     "),      # rounds up into the F range
    (0.0999994, 14, 5, 3, "  0.99999E-001"),
    (-1.234567e-12, 14, 5, 3, " -0.12346E-011"),
    (6.1875e-06, 20, 8, 0, "      0.61875000E-05"),
    (3.14159e120, 20, 8, 0, "      0.31415900+121"),  # 3-digit exponent without Ee drops the E
    (123456.7, 20, 8, 0, "       123456.70    "),
])
def test_g_edit_rules(tio, x, w, d, e, want):
    assert tio.format_g(x, w, d, e) == want


def test_shipped_equalize_rows_come_back_byte_for_byte(tio, golden):
    """equalize.dat '(g20.8,15(i10))' (composition.f90:568-574), comp = 0:
    time, tpc, minexcess(0), deficits, moved, nfree, count_display(0)."""
    for line in golden["text_lines"]["equalize.dat"]:
        f = fields(line, SPECS["equalize.dat"])
        row = [1] + [int(v) for v in f[1:]]
        assert tio.equalize_line(float(f[0]), row) == line
