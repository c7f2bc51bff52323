"""GPU test of gbh_morton_order_noalloc, the entry point for callers that cannot allocate device
memory (their GPU memory belongs to another allocator, or they must not take the synchronisation
cudaMalloc can imply). It must give exactly the Morton keys and sort order that the allocating
path (gbh_accelerations, then gbh_tree_export) gives, call after call: its temporaries live in
one static device array that keeps the previous call's contents.

This file is collected last so that a run stopping at its first failure has already run every
other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from gravitas_gb300 import abi

pytestmark = pytest.mark.gpu
P = abi.ptr
MAX_BODIES = 262144


def state(n, seed):
    rng = np.random.default_rng(seed)
    p = rng.normal(size=(n, 3)) * rng.uniform(0.5, 2.0)
    kind = rng.choice([abi.STAR, abi.DARK_MATTER, abi.GAS], n).astype(np.uint8)
    kind[::101] = abi.BLACK_HOLE
    alive = (rng.random(n) > 0.05).astype(np.uint8)
    return dict(px=p[:, 0].copy(), py=p[:, 1].copy(), pz=p[:, 2].copy(), mass=rng.uniform(0.5, 1.5, n),
                kind=kind, alive=alive)


def test_morton_order_without_allocation_matches_allocating_path():
    torch = pytest.importorskip("torch")
    L = abi.load()
    ctx = abi.Context(0)
    dev = torch.device("cuda:0")
    # two calls in a row, the second smaller, so it runs over the first call's leftovers
    for seed, n in ((1, 200_000), (2, 70_001)):
        s = state(n, seed)
        ax, ay, az = (np.zeros(n) for _ in range(3))
        ctx.call("gbh_accelerations", abi.make_params(0.5, 0.01, 8, False, False, "mixed"), n, P(s["px"]),
                 P(s["py"]), P(s["pz"]), P(s["mass"]), P(s["kind"]), P(s["alive"]), P(ax), P(ay), P(az))
        want = ctx.tree_export()

        d = {k: torch.from_numpy(s[k]).to(dev) for k in ("px", "py", "pz", "kind", "alive")}
        keys = torch.full((n,), -1, dtype=torch.int64, device=dev)
        order = torch.full((n,), -1, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        nstars = np.zeros(1, np.int64)
        err = ctypes.create_string_buffer(256)
        rc = L.gbh_morton_order_noalloc(0, None, n, P(d["px"].data_ptr()), P(d["py"].data_ptr()),
                                        P(d["pz"].data_ptr()), P(d["kind"].data_ptr()), P(d["alive"].data_ptr()),
                                        P(keys.data_ptr()), P(order.data_ptr()), P(nstars), err, 256)
        assert rc == abi.OK, err.value.decode()
        ns = int(nstars[0])
        assert ns == len(want["keys"])
        assert np.array_equal(keys.cpu().numpy()[:ns].view(np.uint64), want["keys"])
        assert np.array_equal(order.cpu().numpy()[:ns], want["order"])
    ctx.close()


def test_morton_order_without_allocation_rejects_too_many_bodies():
    L = abi.load()
    nstars = np.zeros(1, np.int64)
    err = ctypes.create_string_buffer(256)
    rc = L.gbh_morton_order_noalloc(0, None, MAX_BODIES + 1, None, None, None, None, None, None, None, P(nstars),
                                    err, 256)
    assert rc == abi.ERR_ARG
    assert b"262144" in err.value
