"""CPU tests of the .gravitas snapshot codec (internal/save/save.go: gob + gzip).

Go is not available to write reference files, so the gob restatement is pinned to the byte
sequences of the published encoding/gob specification (its integer and float encodings and its
worked example, the stream of Point{22, 33}), and the snapshot layer to the reference's own
save tests (save_test.go:17-52 continue bit-identically after a round trip, :89-100 garbage is
rejected)."""
import gzip
import os

import numpy as np
import pytest

from gravitas_gb300 import ics
from gravitas_gb300 import snapshot as S
from oracle import oracle as O


def test_unsigned_signed_and_float_encodings():
    # encoding/gob: 0 is (00), 7 is (07), 256 is (FE 01 00)
    assert S.enc_uint(0) == b"\x00" and S.enc_uint(7) == b"\x07" and S.enc_uint(256) == b"\xfe\x01\x00"
    # signed: sign in the low bit; -129 = ^128 is sent as the unsigned 257 (FE 01 01)
    assert S.enc_int(-129) == b"\xfe\x01\x01" and S.enc_int(22) == b"\x2c" and S.enc_int(-1) == b"\x01"
    # float64(17) is the unsigned 0x3140 after byte reversal: (FE 31 40)
    assert S.enc_float(17.0) == b"\xfe\x31\x40"
    for v in (0, 1, 127, 128, 255, 256, 2 ** 40 + 5, 2 ** 64 - 1):
        assert S._In(S.enc_uint(v)).uint() == v
    for v in (0, 1, -1, 63, -64, 2 ** 62, -(2 ** 63)):
        assert S._In(S.enc_int(v)).int() == v
    for v in (0.0, -0.0, 1.5, -2.25e-300, 6.02e23, float("inf")):
        got = S._In(S.enc_float(v)).float()
        assert got == v and np.signbit(got) == np.signbit(v)


POINT_STREAM = bytes.fromhex(
    "1fff81030101 05 506f696e74 01ff82 00 0102 010158 0104 00 010159 0104 00 00 00"
    "07ff82 012c 0142 00".replace(" ", ""))


def test_point_example_of_the_gob_specification():
    """type Point struct {X, Y int}; Point{22, 33} -> the 31-byte type definition of Point (id
    65) and the 7-byte value message."""
    point = S.Struct("Point", [("X", S.INT), ("Y", S.INT)])
    assert S.Encoder().encode(point, {"X": 22, "Y": 33}).getvalue() == POINT_STREAM
    assert S.decode(POINT_STREAM) == {"X": 22, "Y": 33}


def test_generic_decode_of_reference_shaped_types():
    """Nested structs, pointers to structs (sent as the struct), maps, arrays, strings, bools,
    GobEncoder bytes (time.Time) and slices of structs, as scene.Spec and save.File hold them."""
    cam = S.Struct("CameraSpec", [("Target", S.Array(S.FLOAT, 3)), ("Distance", S.FLOAT)])
    comp = S.Struct("Component", [("Kind", S.STRING), ("N", S.INT), ("Mass", S.FLOAT)])
    spec = S.Struct("Spec", [("Name", S.STRING), ("Intro", S.Map(S.STRING, S.STRING)), ("Camera", cam),
                             ("Paused", S.BOOL), ("Components", S.Slice(comp)), ("SNDelayMyr", S.Array(S.FLOAT, 2))])
    f = S.Struct("File", [("Format", S.INT), ("Saved", S.Encoded("time.Time")), ("Scene", spec),
                          ("Steps", S.INT), ("PosX", S.Slice(S.FLOAT)), ("Kind", S.BYTES), ("Spins", S.Slice(S.INT))])
    saved = bytes([1, 0, 0, 0, 14, 222, 0, 0, 1, 0, 0, 0, 0, 255, 255])  # a time.Time MarshalBinary value
    v = {"Format": 4, "Saved": saved,
         "Scene": {"Name": "Merger", "Intro": {"school": "two galaxies", "physics": "parabolic"},
                   "Camera": {"Target": [0.0, 1.0, -2.0], "Distance": 40.0}, "Paused": True,
                   "Components": [{"Kind": "disk", "N": 40000, "Mass": 0.4}, {"Kind": "halo", "N": 0, "Mass": 0}],
                   "SNDelayMyr": [3.0, 40.0]},
         "Steps": 0, "PosX": np.array([1.0, -0.5, 2.5e-9]), "Kind": bytes([0, 1, 2]), "Spins": [5, -7]}
    got = S.decode(S.Encoder().encode(f, v).getvalue())
    assert got["Format"] == 4 and got["Saved"] == saved and "Steps" not in got  # zero fields are not sent
    sc = got["Scene"]
    assert sc["Name"] == "Merger" and sc["Intro"] == v["Scene"]["Intro"] and sc["Paused"] is True
    assert list(sc["Camera"]["Target"]) == [0.0, 1.0, -2.0] and sc["Camera"]["Distance"] == 40.0
    assert sc["Components"][0] == {"Kind": "disk", "N": 40000, "Mass": 0.4} and sc["Components"][1] == {"Kind": "halo"}
    assert np.array_equal(got["PosX"], v["PosX"]) and got["Kind"] == bytes([0, 1, 2])
    assert list(got["Spins"]) == [5, -7]


def test_round_trip_keeps_every_bit(tmp_path):
    s = ics.test_disk(2000)
    rng = np.random.default_rng(3)
    acc = [rng.normal(size=len(s["px"])) for _ in range(3)]
    p = os.path.join(tmp_path, "disk" + S.EXTENSION)
    S.save(p, s, {"Dt": 0.004, "Softening": 0.06, "C": 10.0}, time=1.25, steps=312, forces=acc)
    st, params, meta = S.load_state(p)
    for k in ("px", "py", "pz", "vx", "vy", "vz", "mass", "kind"):
        assert np.array_equal(st[k], s[k]), k
    for k, a in zip(("ax", "ay", "az"), acc):
        assert np.array_equal(st[k], a), k
    assert params == {"Dt": 0.004, "Softening": 0.06, "C": 10.0}
    assert meta["Time"] == 1.25 and meta["Steps"] == 312 and meta["forces"] and meta["Format"] == S.FORMAT


def test_save_load_continues_bit_identically(tmp_path):
    """save_test.go:17-52: stepping, saving (with the last forces), loading and stepping on gives
    the trajectory of stepping straight through."""
    s = ics.plummer(3000, seed=4)
    keys = ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az", "mass")
    straight = {k: s[k].copy() for k in keys}
    O.kdk(straight, dt=1e-3, eps=0.01, theta=0.5, leaf=8, nsteps=6, workers=1)
    half = {k: s[k].copy() for k in keys}
    O.kdk(half, dt=1e-3, eps=0.01, theta=0.5, leaf=8, nsteps=3, workers=1)
    p = os.path.join(tmp_path, "run.gravitas")
    S.save(p, half, {"Dt": 1e-3, "Softening": 0.01}, steps=3, forces=(half["ax"], half["ay"], half["az"]))
    st, params, meta = S.load_state(p)
    assert meta["forces"]
    O.kdk(st, dt=params["Dt"], eps=params["Softening"], theta=0.5, leaf=8, nsteps=3, acc_valid=True, workers=1)
    for k in keys:
        assert np.array_equal(st[k], straight[k]), k


def test_garbage_is_rejected(tmp_path):  # save_test.go:89-100
    for i, blob in enumerate((b"not a snapshot", gzip.compress(b"\x05\x03\x01\x02"), gzip.compress(b""),
                              gzip.compress(POINT_STREAM[:20]))):
        p = os.path.join(tmp_path, f"bad{i}.gravitas")
        with open(p, "wb") as f:
            f.write(blob)
        with pytest.raises(S.GobError):
            S.read(p)


def test_saved_forces_satisfy_the_reference_restore_condition(tmp_path):
    """RestoreForces (sim.go:208-212) installs saved forces only when AccX and Rho both hold one
    entry per body; the writer therefore sends Rho (zeros) beside the accelerations."""
    s = ics.plummer(500, seed=6)
    n = len(s["px"])
    p = os.path.join(tmp_path, "f.gravitas")
    S.save(p, s, {"Dt": 1e-3, "Softening": 0.01}, forces=(s["ax"] + 1, s["ay"], s["az"]))
    f = S.read(p)["Forces"]
    assert len(f["AccX"]) == n and len(f["Rho"]) == n and not np.any(f["Rho"])


def test_simulation_save_keeps_only_alive_bodies(tmp_path):
    """The file format has no alive flags (File.State makes every body alive), and the reference
    never saves dead bodies because it compacts them away at once (State.Compact,
    state.go:99-122). Simulation.save writes the alive bodies in state order, with their forces,
    and leaves the in-memory state as it was."""
    from gravitas_gb300.sim import Params, Simulation, State

    d = ics.plummer(400, seed=7)
    st = State.from_dict(d)
    rng = np.random.default_rng(1)
    st.acc_x[:] = rng.normal(size=len(st))
    st.alive[[3, 150, 399]] = 0
    m = Simulation(st, solver=None, params=Params(dt=1e-3, softening=0.01))
    m.acc_valid = True
    p = os.path.join(tmp_path, "dead.gravitas")
    m.save(p)
    got, _, meta = S.load_state(p)
    keep = st.alive.astype(bool)
    assert len(got["px"]) == keep.sum() == 397 and meta["forces"]
    assert np.array_equal(got["px"], st.pos_x[keep]) and np.array_equal(got["ax"], st.acc_x[keep])
    assert np.array_equal(got["kind"], st.kind[keep]) and got["alive"].all()
    assert len(st) == 400 and st.alive.sum() == 397


def test_evolve_watchdog_restates_first_bad(capsys):
    """firstBad (tools/evolve/main.go:185-194): NaN or |v| > 1e6 in the x position, x velocity or x
    acceleration marks a body (infinities included; the y and z components are not looked at, as
    in the reference); the report names the body and every black hole's distance and speed."""
    from gravitas_gb300 import evolve
    from gravitas_gb300.sim import Params, Simulation, State

    st = State.from_dict(ics.plummer(50, seed=2))
    assert evolve.first_bad(st) == -1
    st.pos_y[5] = np.nan  # not a component firstBad reads
    st.vel_z[6] = 1e9
    assert evolve.first_bad(st) == -1
    for arr, v, i in ((st.acc_x, np.nan, 30), (st.vel_x, -2e6, 20), (st.pos_x, np.inf, 9)):
        arr[i] = v
        assert evolve.first_bad(st) == i
    st.pos_x[9] = 1e6  # the bound itself is allowed
    assert evolve.first_bad(st) == 20
    st.kind[40] = 1
    m = Simulation(st, solver=None, params=Params(dt=1e-3))
    evolve.report_bad(m, 20)
    out = capsys.readouterr().out
    assert "body 20" in out and "hole 40" in out
