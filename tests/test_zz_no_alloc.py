"""rd_rasterize_noalloc: the allocation-free rasterize for callers that cannot
allocate GPU memory (an engine whose pool owns the device, a frame loop that
cannot afford cudaMalloc's synchronisation or an out-of-memory failure).  It
must give what the handle-based entry point gives - rd_stage(RASTERIZE) read
back through rd_get_grid - on consecutive calls that reuse its fixed scratch,
and report through rd_rasterize_noalloc_flags what its kernels found.
Collected last so that a run stopping at the first failure has run the rest."""
import ctypes

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def _scene(seed, n, G, radius=0.2):
    rng = np.random.default_rng(seed)
    h = np.float32(1.0 / G)
    d = rng.normal(size=(n, 3))
    d = d / np.linalg.norm(d, axis=1, keepdims=True) * rng.uniform(size=(n, 1)) ** (1 / 3) * radius
    x = (d + 0.5).astype(np.float32)
    v = rng.normal(0, 1.0, (n, 3)).astype(np.float32)
    m = rng.uniform(0.5e-4, 1.5e-4, n).astype(np.float32)
    dinv = 3.0 / float(h) ** 2
    B = (rng.normal(0, 0.3, (n, 9)) / dinv).astype(np.float32)
    return h, x, v, m, B


def _noalloc(pkg, params, x, v, m, B):
    import torch
    xd, vd, md, bd = (torch.from_numpy(a).cuda() for a in (x, v, m, B))
    cells = params.max_i * params.max_j * params.max_k
    out = torch.full((cells, 4), float("nan"), dtype=torch.float32, device="cuda")
    parts = pkg._Particles(x=xd.data_ptr(), v=vd.data_ptr(), B=bd.data_ptr(), FE=None, FP=None, Jp=None,
                           mass=md.data_ptr(), volume=None)
    st = pkg.lib().rd_rasterize_noalloc(ctypes.byref(params), ctypes.byref(parts), out.data_ptr(), None)
    assert st == pkg.RD_OK, pkg.STATUS_NAMES.get(st, st)
    torch.cuda.synchronize()
    flags = ctypes.c_uint32(0xFFFFFFFF)
    assert pkg.lib().rd_rasterize_noalloc_flags(ctypes.byref(flags)) == pkg.RD_OK
    return out.cpu().numpy(), flags.value


def _handle(pkg, params, x, v, m, B):
    with pkg.Simulation(params) as sim:
        sim.set_particles(x, v, m, B=B)
        sim.stage("rasterize")
        grid = sim.get_grid()
        flags = sim.flags()
    return grid, flags


def test_noalloc_rasterize_matches_handle_rasterize(built_pkg):
    pkg = built_pkg
    for seed, n, G in ((0, 5000, 32), (1, 20000, 48)):  # two calls in a row, different sizes
        h, x, v, m, B = _scene(seed, n, G)
        params = pkg.make_params(G, G, G, n, float(h))
        grid, hflags = _handle(pkg, params, x, v, m, B)
        mom = grid["mass"][:, None].astype(np.float64) * grid["vel"]
        got, flags = _noalloc(pkg, params, x, v, m, B)
        assert rel(got[:, 0], grid["mass"]) < 1e-6
        assert rel(got[:, 1:], mom) < 1e-5
        assert float(np.abs(got[grid["mass"] == 0]).max()) == 0.0
        assert flags == 0 and hflags == 0


def test_noalloc_partial_blocks_and_walls(built_pkg):
    """Grid sizes that are not multiples of the 4-cell sort block (the last
    block of each axis is partial), with particles near every wall: some
    stencils reach past the grid (those nodes are dropped and
    RD_FLAG_OUT_OF_DOMAIN is raised, as the handle raises it), and a call
    after such a call starts with clear flags."""
    pkg = built_pkg
    for seed, G in ((2, 30), (3, 37)):
        h, x, v, m, B = _scene(seed, 6000, G, radius=0.3)
        rng = np.random.default_rng(seed + 100)
        k = 200  # particles within two cells of a wall, some within one
        w = rng.integers(0, 3, k)
        side = rng.integers(0, 2, k)
        x[:k] = rng.uniform(3.0 * h, (G - 3) * h, (k, 3)).astype(np.float32)
        depth = rng.uniform(0.2, 2.0, k) * float(h)
        x[np.arange(k), w] = np.where(side == 0, depth, G * float(h) - depth - float(h)).astype(np.float32)
        params = pkg.make_params(G, G, G, len(m), float(h))
        grid, hflags = _handle(pkg, params, x, v, m, B)
        got, flags = _noalloc(pkg, params, x, v, m, B)
        assert hflags & pkg.FLAG_OUT_OF_DOMAIN
        assert flags == hflags, (flags, hflags)
        mom = grid["mass"][:, None].astype(np.float64) * grid["vel"]
        assert rel(got[:, 0], grid["mass"]) < 1e-6
        assert rel(got[:, 1:], mom) < 1e-5
        assert float(np.abs(got[grid["mass"] == 0]).max()) == 0.0
        # every particle inside the domain again: the next call reports nothing
        h2, x2, v2, m2, B2 = _scene(seed, 3000, G)
        p2 = pkg.make_params(G, G, G, len(m2), float(h2))
        _, flags2 = _noalloc(pkg, p2, x2, v2, m2, B2)
        assert flags2 == 0


def test_noalloc_rejects_sizes_beyond_its_scratch(built_pkg):
    pkg = built_pkg
    L = pkg.lib()
    dummy = pkg._Particles(x=1, v=1, B=None, FE=None, FP=None, Jp=None, mass=1, volume=None)
    for dims, n in (((128, 128, 128), 1000), ((64, 64, 64), 70000)):
        p = pkg.make_params(*dims, n, 1.0 / dims[0])
        assert L.rd_rasterize_noalloc(ctypes.byref(p), ctypes.byref(dummy), 1, None) == pkg.RD_TOO_LARGE
    p = pkg.make_params(32, 32, 32, 10, 1 / 32, precision=pkg.RD_FP64)
    assert L.rd_rasterize_noalloc(ctypes.byref(p), ctypes.byref(dummy), 1, None) == pkg.RD_NOT_SUPPORTED
