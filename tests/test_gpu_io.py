"""GPU: the device text I/O against the reference's formats.  Expected
values come from Python's own conversions (float() is correctly rounded as
strtod is; '%12.6f' rounds the binary value exactly as printf does), with
the reference's line rules (GridObservation.hpp:395-474, SimpleState.hpp:
160-188, 248-263) restated below."""
import math

import numpy as np
import pytest
import torch

import oracle.bind as ob
from metada_gb300 import kernels as K
from metada_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

HEADER = "Time Z   Y   X   ZNU      XLONG_U    XLAT_U     Simple"
SEP = "-" * 80


def _ref_parse_obs(text: str, missing: float):
    """The loop of GridObservation::loadFromFile on well-formed tokens."""
    out = []
    header = started = False
    for line in text.split("\n"):
        if not line:
            continue
        if "Time" in line and "XLONG_U" in line:
            header = True
            continue
        if "---" in line and not line.strip("- \t"):
            if header:
                started = True
            continue
        if not started:
            continue
        parts = line.split()
        try:
            t, z, y, x = (int(v) for v in parts[:4])
            znu, lon, lat, val = (float(v) for v in parts[4:8])
        except (ValueError, IndexError):
            continue
        if len(parts) < 8:
            continue
        if val != missing:
            out.append((x, y, z, znu, lon, lat, val))
    return out


def test_parse_grid_obs_written_by_the_reference_writer(dev):
    c = syn.global_etkf_grid(case=9)
    import tempfile
    from pathlib import Path

    with tempfile.TemporaryDirectory() as td:
        p = Path(td) / "obs.txt"
        syn.write_grid_obs(p, c.obs_xy, c.yo)
        text = p.read_bytes()
    xyz, vals = K.parse_grid_obs(text)
    want = _ref_parse_obs(text.decode(), -999.0)
    assert xyz.shape[0] == len(want) == len(c.yo)
    w = np.array(want)
    assert np.array_equal(xyz.cpu().numpy(), w[:, :3].astype(np.int32))
    assert np.array_equal(vals.cpu().numpy(), w[:, 3:])


def test_parse_grid_obs_line_rules_and_number_forms(dev):
    lines = [
        "0 1 2 3 0.5 1.0 2.0 9.0",          # before any header: ignored
        HEADER,
        "0 1 2 3 0.5 1.0 2.0 8.0",          # header but no separator yet: ignored
        SEP,
        "0    1   3   4  0.7035   -82.7143   32.6471     0.2052",
        "",
        "0\t1\t3\t9\t0.7035\t-79.8571\t32.6471\t-999.0",   # missing value: dropped
        "0 1 5 6 .5 +1.25 -0.0 1e-3",
        "0 1 5 7 7.0e+1 1E2 3.5E-2 -0.0",
        "0 1 5 8 0.1 0.2 0.3 123456789012345678901234.5",    # 25 digits: both 19-digit bounds round alike
        "0 1 5 9 0.1 0.2 0.3 4.9e-324",                      # subnormal: host path
        "bad line with words",
        "0 1 5",                                             # too few fields
        "0 1 5 10 0.25 0.5 0.75 1.5\r",                      # CRLF line
        SEP,                                                 # later separators: skipped
        HEADER,
        "0 1 6 0 1 2 3 4 trailing tokens are ignored",
    ]
    text = ("\n".join(lines) + "\n").encode()
    xyz, vals = K.parse_grid_obs(text)
    want = [
        (4, 3, 1, 0.7035, -82.7143, 32.6471, 0.2052),
        (6, 5, 1, 0.5, 1.25, -0.0, 1e-3),
        (7, 5, 1, 70.0, 100.0, 0.035, -0.0),
        (8, 5, 1, 0.1, 0.2, 0.3, float("123456789012345678901234.5")),
        (9, 5, 1, 0.1, 0.2, 0.3, 4.9e-324),
        (10, 5, 1, 0.25, 0.5, 0.75, 1.5),
        (0, 6, 1, 1.0, 2.0, 3.0, 4.0),
    ]
    w = np.array(want)
    assert np.array_equal(xyz.cpu().numpy(), w[:, :3].astype(np.int32))
    got = vals.cpu().numpy()
    assert np.array_equal(got, w[:, 3:])
    assert math.copysign(1.0, got[1, 2]) < 0 and math.copysign(1.0, got[2, 3]) < 0  # -0.0 kept
    assert K.last_io_host_items() == 1  # only the subnormal's line went to the host


@pytest.mark.parametrize("nx,ny", [(36, 18), (360, 180)])
def test_state_round_trip(dev, nx, ny):
    g = np.random.default_rng(nx)
    v = g.standard_normal(nx * ny) * 10.0 ** g.integers(-7, 9, nx * ny)
    v[:8] = [0.0078125, -0.0078125, 2.5e-7, -2.5e-7, -0.0, 0.5e-6, 1.0 / 3.0, 2.0 ** 60]  # ties, -0, host path
    text = K.format_state(torch.tensor(v, device=dev), nx, ny)
    rows = [" ".join("%12.6f" % x for x in v[y * nx:(y + 1) * nx]) for y in range(ny)]
    want = ("\n".join(rows) + "\n").encode()
    assert text == want
    back = K.parse_values(text).cpu().numpy()
    assert np.array_equal(back, np.array([float(t) for t in want.split()]))
    assert np.array_equal(back, ob.parse_values(text))  # the reference's own extraction loop


def test_parse_values_long_lines_every_line_mode(dev):
    # Lines of hundreds of values (one warp per line): regular lines, lines
    # whose tokens are not whole numbers ("1.5-2.5", "1.5.5": read by the
    # sequential loop), a failed extraction mid-line, a number for the host,
    # CRLF endings, tabs and runs of blanks.
    g = np.random.default_rng(7)

    def vals(n):
        return ["%.6f" % x for x in g.standard_normal(n) * 100.0]

    lines = [
        "  " + " ".join(vals(400)) + "   ",
        " ".join(vals(300) + ["1.5-2.5"] + vals(200)),
        " ".join(vals(250) + ["abc"] + vals(100)),
        " ".join(vals(300) + ["12.000000000000000000001"] + vals(50)),
        "\t".join(vals(300)) + "\r",
        "  ".join(vals(100) + ["1e5", "-.5", "+3.", "5E-3", "1.5.5", "-0.0"] + vals(100)),
        " ".join(vals(600) + ["1e"]),
        " ".join(vals(200) + ["7.5e+"] + vals(20)),
        "",
        "42",
    ]
    text = ("\n".join(lines) + "\n").encode()
    assert len(text) >= 256 * len(lines)
    got = K.parse_values(text).cpu().numpy()
    want = ob.parse_values(text)
    assert got.shape == want.shape and np.array_equal(got, want)
    assert np.array_equal(np.signbit(got), np.signbit(want))


def test_parse_values_stops_a_line_at_the_first_failed_extraction(dev):
    text = b"1.5 2.5 x 3.5\n  4 5e1\n\n-0.25 .75 7.\n1 2 3 4 5 6 7 8 9 10 11 12.000000000000000000001\n"
    got = K.parse_values(text).cpu().numpy()
    want = [1.5, 2.5, 4.0, 50.0, -0.25, 0.75, 7.0] + [float(i) for i in range(1, 12)] + [12.000000000000000000001]
    assert np.array_equal(got, np.array(want))
    assert np.array_equal(got, ob.parse_values(text))


def test_save_ensemble_writes_the_reference_text(dev, tmp_path):
    """saveEnsemble on a SimpleGeometry: the mean and every member as the
    reference's "%12.6f" rows (SimpleState::saveToFile), from the device."""
    from metada_gb300 import algorithms as A

    nx, ny, k = 36, 18, 5
    c = syn.global_etkf_grid(nx=nx, ny=ny, k=k, p=64, case=71)
    X = c.X.copy()
    X[0, :6] = [0.0078125, -0.0078125, -0.0, 2.5e-7, 2.0 ** 60, 1.0 / 3.0]  # ties, -0, host path
    ens = A.Ensemble(X, A.SimpleGeometry(nx, ny), device=dev)
    obs = A.Observation(c.yo, c.sigma_o, grid_xy=c.obs_xy, device=dev)
    base = tmp_path / "out" / "analysis"
    A.ETKF(ens, obs, A.ObsOperator(), {"inflation": 1.05, "output_base_file": str(base)}).saveEnsemble()

    def text(v):
        return ("\n".join(" ".join("%12.6f" % x for x in v[y * nx:(y + 1) * nx]) for y in range(ny)) + "\n").encode()

    assert (tmp_path / "out" / "analysis_mean.txt").read_bytes() == text(ens.Mean())
    for i in range(k):
        assert (tmp_path / "out" / f"analysis_member_{i}.txt").read_bytes() == text(X[i])


def _number_strings(rng, n, digits_lo, digits_hi):
    """Decimal strings of normal doubles in the forms std::istream reads:
    random significant digits, a decimal point anywhere (or none), an
    optional exponent (e/E, signed), an optional sign."""
    out = []
    for _ in range(n):
        nd = int(rng.integers(digits_lo, digits_hi + 1))
        digs = str(int(rng.integers(1, 10))) + "".join(str(d) for d in rng.integers(0, 10, nd - 1))
        point = int(rng.integers(0, nd + 1))
        body = digs[:point] + "." + digs[point:] if point < nd else digs
        if body.startswith("."):
            body = "0" + body if rng.random() < 0.5 else body
        mag = point  # decimal exponent of the leading digit + 1
        e = int(rng.integers(-300 - mag + 2, 300 - mag))
        s = body
        if rng.random() < 0.8:
            s += ("e" if rng.random() < 0.5 else "E") + (("+" if rng.random() < 0.3 else "") if e >= 0 else "") + str(e)
        if rng.random() < 0.3:
            s = "-" + s
        out.append(s)
    return out


def _bits(a):
    return np.asarray(a, dtype=np.float64).view(np.uint64)


def test_parse_values_decides_normal_numbers_on_the_device(dev):
    """Numbers of 1 to 19 significant digits whose values are normal doubles,
    with exponents across the whole range: every one is converted on the
    device (Clinger's path or Eisel-Lemire), bit for bit as Python's
    correctly rounded float(); none goes to the host."""
    rng = np.random.default_rng(11)
    toks = _number_strings(rng, 40_000, 1, 19)
    text = "\n".join(" ".join(toks[i:i + 10]) for i in range(0, len(toks), 10)).encode() + b"\n"
    got = K.parse_values(text).cpu().numpy()
    assert K.last_io_host_items() == 0
    want = np.array([float(t) for t in toks])
    assert np.array_equal(_bits(got), _bits(want))


def test_parse_values_long_mantissas_and_the_host_rest(dev):
    """20 to 40 significant digits: decided on the device when the two
    19-digit bounds round alike (nearly always), otherwise by the host; a
    line with a subnormal result goes to the host.  Every value bit for bit
    as float()."""
    rng = np.random.default_rng(12)
    toks = _number_strings(rng, 20_000, 20, 40)
    lines = [" ".join(toks[i:i + 10]) for i in range(0, len(toks), 10)]
    lines.append("1.5 4.9e-324 2.5")
    text = ("\n".join(lines) + "\n").encode()
    got = K.parse_values(text).cpu().numpy()
    host = K.last_io_host_items()
    assert 1 <= host <= len(lines) // 20
    want = np.array([float(t) for t in toks] + [1.5, 4.9e-324, 2.5])
    assert np.array_equal(_bits(got), _bits(want))
