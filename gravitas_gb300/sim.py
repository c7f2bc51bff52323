"""Host-side mirror of gravitas' force and step API over the C-ABI.

Names follow the reference: State is sim.State (internal/sim/state.go:33-52) as SoA numpy
arrays, Params the fields of sim.Params the path reads (sim.go:9-23), Solver is bh.Solver
(internal/sim/bh/bh.go:28-102, potential.go:12-42), DirectSolver is direct.Solver
(internal/sim/direct/direct.go:14-48) and Simulation.step is Simulation.Step (sim.go:248-288)
for states without black holes or hydro. Every computation runs in libgbh.so on the GPU.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import abi

DEFAULT_THETA = 0.9   # bh.go:14-16
LEAF_SIZE = 24        # bh.go:17-19
DIAG_THETA = 0.9      # bh.go:20-23

_F = ("pos_x", "pos_y", "pos_z", "vel_x", "vel_y", "vel_z", "acc_x", "acc_y", "acc_z", "mass")


@dataclass
class Params:
    dt: float = 0.0
    softening: float = 0.0
    c: float = 0.0
    dark_matter_off: bool = False


@dataclass
class State:
    """Bodies as struct-of-arrays (FP64 positions, velocities, accelerations, masses)."""
    pos_x: np.ndarray = field(default_factory=lambda: np.zeros(0))
    pos_y: np.ndarray = field(default_factory=lambda: np.zeros(0))
    pos_z: np.ndarray = field(default_factory=lambda: np.zeros(0))
    vel_x: np.ndarray = field(default_factory=lambda: np.zeros(0))
    vel_y: np.ndarray = field(default_factory=lambda: np.zeros(0))
    vel_z: np.ndarray = field(default_factory=lambda: np.zeros(0))
    acc_x: np.ndarray = field(default_factory=lambda: np.zeros(0))
    acc_y: np.ndarray = field(default_factory=lambda: np.zeros(0))
    acc_z: np.ndarray = field(default_factory=lambda: np.zeros(0))
    mass: np.ndarray = field(default_factory=lambda: np.zeros(0))
    kind: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint8))
    alive: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint8))

    def __post_init__(self):
        for f in _F:
            setattr(self, f, np.ascontiguousarray(getattr(self, f), np.float64))
        self.kind = np.ascontiguousarray(self.kind, np.uint8)
        self.alive = np.ascontiguousarray(self.alive, np.uint8)

    def __len__(self):
        return len(self.mass)

    @classmethod
    def from_dict(cls, d: dict) -> "State":
        n = len(d["mass"])
        return cls(d["px"].copy(), d["py"].copy(), d["pz"].copy(), d.get("vx", np.zeros(n)).copy(),
                   d.get("vy", np.zeros(n)).copy(), d.get("vz", np.zeros(n)).copy(), np.zeros(n), np.zeros(n),
                   np.zeros(n), d["mass"].copy(), d.get("kind", np.zeros(n, np.uint8)).copy(),
                   d.get("alive", np.ones(n, np.uint8)).copy())

    def acc(self) -> np.ndarray:
        return np.stack([self.acc_x, self.acc_y, self.acc_z], axis=1)


_ctx = None


def default_context() -> abi.Context:
    global _ctx
    if _ctx is None:
        _ctx = abi.Context(0)
    return _ctx


class Solver:
    """bh.Solver: Theta (0 means 0.9), MonopoleOnly, the walk variant and the leaf size."""

    def __init__(self, theta: float = 0.0, monopole_only: bool = False, walk: str = "mixed",
                 leaf_size: int = LEAF_SIZE, ctx: abi.Context | None = None):
        self.theta, self.monopole_only, self.walk, self.leaf_size = theta, monopole_only, walk, leaf_size
        self.ctx = ctx or default_context()

    def params(self, p: Params) -> abi.Params:
        return abi.make_params(self.theta, p.softening, self.leaf_size, self.monopole_only, p.dark_matter_off,
                               self.walk, c=p.c)

    def accelerations(self, s: State, p: Params) -> None:
        """Fills s.acc_* (bh.go:76-102): holes get 0, dead bodies keep their entries."""
        P = abi.ptr
        self.ctx.call("gbh_accelerations", self.params(p), len(s), P(s.pos_x), P(s.pos_y), P(s.pos_z), P(s.mass),
                      P(s.kind), P(s.alive), P(s.acc_x), P(s.acc_y), P(s.acc_z))

    def potential_energy(self, s: State, p: Params) -> float:
        """Tree estimate of the potential energy at min(theta, 0.9) (potential.go:12-42)."""
        P = abi.ptr
        u = np.zeros(1)
        self.ctx.call("gbh_potential_energy", self.params(p), len(s), P(s.pos_x), P(s.pos_y), P(s.pos_z),
                      P(s.mass), P(s.kind), P(s.alive), float(p.c), P(u))
        return float(u[0])

    def last_timings(self) -> dict:
        return self.ctx.timings()


class DirectSolver:
    """direct.Solver: the O(N^2) FP64 sum (direct.go:18-48), on the GPU."""

    def __init__(self, ctx: abi.Context | None = None):
        self.ctx = ctx or default_context()

    def accelerations(self, s: State, p: Params, targets=None) -> np.ndarray | None:
        P = abi.ptr
        par = abi.make_params(0.0, p.softening, 0, False, p.dark_matter_off, "fp64")
        if targets is None:
            self.ctx.call("gbh_direct_accelerations", par, len(s), P(s.pos_x), P(s.pos_y), P(s.pos_z), P(s.mass),
                          P(s.kind), None, 0, P(s.acc_x), P(s.acc_y), P(s.acc_z))
            return None
        t = np.ascontiguousarray(targets, np.int64)
        out = np.zeros((3, len(t)))
        self.ctx.call("gbh_direct_accelerations", par, len(s), P(s.pos_x), P(s.pos_y), P(s.pos_z), P(s.mass),
                      P(s.kind), P(t), len(t), P(out[0]), P(out[1]), P(out[2]))
        return out.T.copy()


class Simulation:
    """Simulation.Step (sim.go:248-288) without hydro: the KDK step, or with alive black holes
    the hole-aware split step (c = 0)."""

    def __init__(self, state: State, solver: Solver, params: Params):
        self.state, self.solver, self.params = state, solver, params
        self.time, self.steps = 0.0, 0
        self.acc_valid = False

    def step(self, n: int = 1) -> None:
        s, P = self.state, abi.ptr
        self.solver.ctx.call("gbh_step_kdk", self.solver.params(self.params), float(self.params.dt), int(n),
                             int(self.acc_valid), len(s), P(s.pos_x), P(s.pos_y), P(s.pos_z), P(s.vel_x),
                             P(s.vel_y), P(s.vel_z), P(s.acc_x), P(s.acc_y), P(s.acc_z), P(s.mass), P(s.kind),
                             P(s.alive))
        self.acc_valid = True
        self.time += n * self.params.dt
        self.steps += n

    def save(self, path: str) -> None:
        """A .gravitas snapshot of the run (save.Capture + Write, save.go:66-146), with the last
        forces when they are valid, so that a loaded run continues bit-identically.

        The file format has no alive flags: File.State (save.go:84-111) makes every saved body
        alive. The reference never holds dead bodies when it saves, because accretion and
        collapse remove them at once (State.Compact, state.go:99-122). So the snapshot holds the
        alive bodies only, in state order, as Compact leaves them; the Simulation itself is not
        changed."""
        from . import snapshot
        s = self.state
        keep = s.alive.astype(bool) if len(s.alive) == len(s) else np.ones(len(s), bool)
        sel = (lambda a: a) if keep.all() else (lambda a: np.ascontiguousarray(a[keep]))
        state = {"px": sel(s.pos_x), "py": sel(s.pos_y), "pz": sel(s.pos_z), "vx": sel(s.vel_x),
                 "vy": sel(s.vel_y), "vz": sel(s.vel_z), "mass": sel(s.mass), "kind": sel(s.kind)}
        params = {"Dt": self.params.dt, "Softening": self.params.softening, "C": self.params.c,
                  "DarkMatterOff": self.params.dark_matter_off}
        forces = (sel(s.acc_x), sel(s.acc_y), sel(s.acc_z)) if self.acc_valid else None
        snapshot.save(path, state, params, time=self.time, steps=self.steps, forces=forces)

    @classmethod
    def load(cls, path: str, solver: "Solver") -> "Simulation":
        """A run restored from a snapshot (File.Restore, save.go:113-121)."""
        from . import snapshot
        st, params, meta = snapshot.load_state(path)
        state = State(st["px"], st["py"], st["pz"], st["vx"], st["vy"], st["vz"], st["ax"], st["ay"], st["az"],
                      st["mass"], st["kind"], st["alive"])
        m = cls(state, solver, Params(dt=params.get("Dt", 0.0), softening=params.get("Softening", 0.0),
                                      c=params.get("C", 0.0), dark_matter_off=bool(params.get("DarkMatterOff", False))))
        m.time, m.steps, m.acc_valid = float(meta["Time"]), int(meta["Steps"]), bool(meta["forces"])
        return m


def trajectory_loss_gradient(state: dict, targets: np.ndarray, dt: float, softening: float, nsteps: int,
                             every: int = 50, precision: int = abi.ADJ_FP32, ctx: abi.Context | None = None,
                             force: int = abi.ADJ_DIRECT, theta: float = 0.0, leaf: int = 0):
    """Loss L = mean_i |x_i(T) - target_i|^2 after nsteps KDK steps of the softened direct-sum
    dynamics (force=abi.ADJ_TREE: the Barnes-Hut force at theta and leaf size leaf, its lists
    frozen per step), and its gradient with respect to the initial positions, velocities (n x 3
    each) and masses, through the adjoint pair gbh_fwd_save / gbh_bwd (checkpoints every `every`
    steps, recomputation in between). Returns (loss, dx0, dv0, dm)."""
    ctx = ctx or default_context()
    x0 = np.stack([state["px"], state["py"], state["pz"]], 1)
    v0 = np.stack([state["vx"], state["vy"], state["vz"]], 1)
    xT, _ = ctx.fwd_save(x0, v0, state["mass"], dt, softening, nsteps, every, precision, force, theta, leaf)
    r = xT - targets
    n = len(r)
    loss = float(np.sum(r * r) / n)
    dx, dv, dm = ctx.bwd(2.0 * r / n, None)
    return loss, dx, dv, dm
