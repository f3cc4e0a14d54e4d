"""The reference's on-disk formats, byte for byte, on the host (no device).

BulkQuantitiesInTime rows (diagnostics/methods/BulkQuantitiesInTime.java:105-115):
DecimalFormat("0.################E0") of each value, tab separated.  The
expected strings are written out here from the DecimalFormat rules: the
mantissa takes the shortest round-trip digits of the double (DigitList.set),
one integer digit, no '+' in the exponent.

EnergyDensity files (diagnostics/methods/EnergyDensity.java:15-31,56-100):
int32 D, int32 N[D], then N^D float64, big-endian (DataOutputStream), one file
per output named base_<counter>.<extension>, the first output at step
max(Math.round(startTime/dt), 1) and then every Math.round(interval/dt) steps.
"""
import struct
import types

import numpy as np

from openpixi_gb300.diagnostics import BulkQuantitiesInTime, EnergyDensity, java_round, java_sci


def test_java_sci_digits():
    cases = {0.1: "1E-1", 1234.5: "1.2345E3", 0.05: "5E-2", 100.0: "1E2", -2.5e-10: "-2.5E-10", 0.0: "0E0",
             1.0 / 3.0: "3.333333333333333E-1", 2.0 / 3.0: "6.666666666666666E-1", 1e-14: "1E-14",
             6.02214076e23: "6.02214076E23", 1.2345678901234567e19: "1.2345678901234567E19",
             -1.0: "-1E0", 4 * 0.05: "2E-1", 0.30000000000000004: "3.0000000000000004E-1",
             1.7976931348623157e308: "1.7976931348623157E308"}
    for v, want in cases.items():
        assert java_sci(v) == want, (v, java_sci(v), want)


def test_java_round():
    assert [java_round(v) for v in (2.5, -2.5, 0.5, -0.5, 1.4999999999999998, 0.49999999999999994, 3.0)] == \
        [3, -2, 1, 0, 1, 0, 3]


def test_bulk_quantities_row_bytes(tmp_path):
    d = BulkQuantitiesInTime(str(tmp_path / "bulk.txt"), 0.05)
    d.initialize(types.SimpleNamespace(getTimeStep=lambda: 0.05))
    o = types.SimpleNamespace(e2_total=1.5, b2_total=0.25, px=0.1, py=-0.2, pz=0.30000000000000004,
                              gauss=1e-14, rho2=0.0)
    d.record(o, 4)
    d.record(types.SimpleNamespace(e2_total=1.0 / 3.0, b2_total=1234.5, px=-2.5e-10, py=6.02214076e23, pz=0.05,
                                   gauss=0.0, rho2=100.0), 7)
    raw = (tmp_path / "bulk.txt").read_bytes()
    assert raw == (b"#time \t E^2 \t B^2 \t P_x \t P_y \t P_z \t G \t rho^2\n"
                   b"2E-1\t1.5E0\t2.5E-1\t1E-1\t-2E-1\t3.0000000000000004E-1\t1E-14\t0E0\n"
                   b"3.5000000000000003E-1\t3.333333333333333E-1\t1.2345E3\t-2.5E-10\t6.02214076E23\t5E-2\t0E0\t1E2\n")


class _Grid:
    dims = (3, 2, 4)

    def __init__(self):
        self.calls = 0

    def energy_density(self):
        self.calls += 1
        return np.arange(24, dtype=np.float64) * 0.1 - 1.0 + self.calls


def _read(path):
    raw = open(path, "rb").read()
    D = struct.unpack(">i", raw[:4])[0]
    N = struct.unpack(f">{D}i", raw[4:4 + 4 * D])
    body = np.frombuffer(raw[4 + 4 * D:], dtype=">f8")
    return D, N, body


def test_energy_density_file_round_trip(tmp_path):
    sub = tmp_path / "out"
    sub.mkdir()
    e = EnergyDensity(str(sub / "eps.dat"), 0.1, 0.1)
    e.initialize(types.SimpleNamespace(getTimeStep=lambda: 0.05))
    assert (e.firstStep, e.step) == (2, 2)
    g = _Grid()
    for step in range(7):
        e.calculate(g, [], step)
    # outputs at steps 2, 4, 6 (step 0 is before the first output step)
    assert sorted(p.name for p in sub.iterdir()) == ["eps_1.dat", "eps_2.dat", "eps_3.dat"]
    for k in (1, 2, 3):
        D, N, body = _read(sub / f"eps_{k}.dat")
        assert D == 3 and N == (3, 2, 4)
        assert np.array_equal(body, np.arange(24) * 0.1 - 1.0 + k)
    raw = (sub / "eps_1.dat").read_bytes()
    assert raw[:16] == bytes([0, 0, 0, 3, 0, 0, 0, 3, 0, 0, 0, 2, 0, 0, 0, 4]) and len(raw) == 16 + 24 * 8
    # a name without an extension keeps the dot (FilenameUtils.getExtension is "")
    e2 = EnergyDensity(str(sub / "plain"), 0.0, 0.05)
    e2.initialize(types.SimpleNamespace(getTimeStep=lambda: 0.05))
    e2.calculate(_Grid(), [], 1)
    assert (sub / "plain_1.").exists()
