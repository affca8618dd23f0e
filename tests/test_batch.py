"""Batched fused RK3 over uneven cases: work-list layout (CPU) and parity with
the single-case fused path, CUDA-graph replay and autotuning (GPU)."""
import math

import numpy as np
import pytest
import torch

from tests.cases import quadrant_prims


def test_worklist_layout_covers_every_tile_once():
    from jaxfluids_gb300.batch import build_worklist
    cells = [(64, 64, 1), (40, 24, 1), (128, 128, 1), (17, 33, 1)]
    n, tiles, offsets, wl, total = build_worklist(cells, (16, 32, 1))
    assert total == sum(5 * a * b for a, b, _ in cells)
    assert list(offsets) == [0, 5 * 64 * 64, 5 * 64 * 64 + 5 * 40 * 24, 5 * 64 * 64 + 5 * 40 * 24 + 5 * 128 * 128]
    assert tiles.tolist() == [[4, 2, 1], [3, 1, 1], [8, 4, 1], [2, 2, 1]]
    seen = {(int(c), int(k)) for c, k in wl}
    assert len(seen) == len(wl) == sum(int(t.prod()) for t in tiles)
    assert wl[0][0] == 2  # largest case first


def _configs(sides, **kw):
    from jaxfluids_gb300 import CaseConfig
    return [CaseConfig(cells=(a, b, 1), bc={f: "ZEROGRADIENT" for f in ("east", "west", "north", "south")}, **kw)
            for a, b in sides]


def _cons(cfg, seed):
    from oracle import jf_oracle as O
    q = quadrant_prims(cfg.cells[0], cfg.cells[1], seed=seed)
    P = torch.stack([q[0], q[1], q[2], torch.zeros_like(q[0]), q[3]])
    return O.cons_from_prims(P, cfg.gamma)


SIDES = [(16, 16), (48, 48), (24, 40), (32, 32), (40, 24), (64, 64)]


SCHEMES = [dict(), dict(recon="WENO5-JS", riemann="HLL"), dict(recon="TENO5", riemann="RUSANOV"),
           dict(recon="WENO3-Z"), dict(recon="WENO3-JS", riemann="HLL"), dict(riemann="HLL", signal_speed="DAVIS"),
           dict(recon_var="CHAR-PRIMITIVE", frozen_state="ROE", riemann="HLL"), dict(recon="MINMOD-AD", riemann="HLL")]


@pytest.mark.gpu
@pytest.mark.parametrize("kw", SCHEMES, ids=["-".join(str(v) for v in s.values()) or "weno5z-hllc" for s in SCHEMES])
def test_batched_steps_equal_single_case_steps(kw):
    from jaxfluids_gb300 import BatchedRK3, FusedRK3, build
    build.build()
    cfgs = _configs(SIDES, **kw)
    states = [_cons(c, 100 + i) for i, c in enumerate(cfgs)]
    batch = BatchedRK3(cfgs)
    batch.set_states([s.cuda() for s in states])
    batch.advance(5)
    for i, c in enumerate(cfgs):
        f = FusedRK3(c)
        f.set_state(states[i].cuda())
        f.advance(5)
        torch.cuda.synchronize()
        assert torch.equal(batch.case_view(i), f.cons), i
        assert batch.dt[i].item() == f.dt.item() and batch.t[i].item() == f.t.item()


GEOMETRIES = [
    # 3-D periodic cases of different sizes (the last tile of a periodic line
    # holds no closing face), smooth random-phase states
    ("3d-periodic", [(12, 16, 10), (16, 16, 16), (8, 12, 20)], "PERIODIC", (8, 8, 8)),
    # 2-D: periodic along x, zero-gradient along y
    ("2d-mixed", [(40, 24, 1), (16, 48, 1), (33, 17, 1)], {"east": "PERIODIC", "west": "PERIODIC",
                                                             "north": "ZEROGRADIENT", "south": "ZEROGRADIENT"},
     (16, 16, 1)),
    # 1-D zero-gradient lines of uneven length
    ("1d-zg", [(200, 1, 1), (77, 1, 1), (256, 1, 1)], {"east": "ZEROGRADIENT", "west": "ZEROGRADIENT"},
     (64, 1, 1)),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,cells,bc,tile", GEOMETRIES, ids=[g[0] for g in GEOMETRIES])
def test_batched_geometries_equal_single_case_steps(name, cells, bc, tile):
    """1-D to 3-D cases, periodic and zero-gradient lines, tiles that do not
    divide the cells: every batched case advances bitwise like itself alone."""
    from jaxfluids_gb300 import BatchedRK3, CaseConfig, FusedRK3, build
    from tests.cases import generic_cons
    build.build()
    faces = ("east", "west", "north", "south", "top", "bottom")
    cfgs = []
    for c in cells:
        b = dict(bc) if isinstance(bc, dict) else {f: bc for f, a in zip(faces, (0, 0, 1, 1, 2, 2)) if c[a] > 1}
        cfgs.append(CaseConfig(cells=c, bc=b))
    states = [generic_cons(c, seed=10 + i) for i, c in enumerate(cells)]
    batch = BatchedRK3(cfgs, tile=tile, threads=128)
    batch.set_states([s.cuda() for s in states])
    batch.advance(4)
    for i, c in enumerate(cfgs):
        f = FusedRK3(c)
        f.set_state(states[i].cuda())
        f.advance(4)
        torch.cuda.synchronize()
        assert torch.equal(batch.case_view(i), f.cons), i
        assert batch.dt[i].item() == f.dt.item() and batch.t[i].item() == f.t.item()


@pytest.mark.gpu
def test_graph_replay_and_retile_match_eager():
    from jaxfluids_gb300 import BatchedRK3, build
    build.build()
    cfgs = _configs(SIDES)
    states = [_cons(c, 200 + i).cuda() for i, c in enumerate(cfgs)]
    eager = BatchedRK3(cfgs)
    eager.set_states(states)
    eager.advance(4)
    graphed = BatchedRK3(cfgs, tile=(8, 64, 1), threads=128, ctas=37)
    graphed.set_states(states)
    g = graphed.capture(3)      # runs 1 eager step, then captures 3
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(graphed.cons, eager.cons)
    assert torch.equal(graphed.dt_states, eager.dt_states)


@pytest.mark.gpu
def test_autotune_keeps_the_state():
    from jaxfluids_gb300 import BatchedRK3, autotune, build
    build.build()
    cfgs = _configs(SIDES[:3])
    batch = BatchedRK3(cfgs)
    batch.set_states([_cons(c, 300 + i).cuda() for i, c in enumerate(cfgs)])
    before = batch.cons.clone()
    res = autotune(batch, candidates=[((16, 32, 1), 256, 152), ((8, 64, 1), 128, 304), ((32, 16, 1), 256, 76)])
    assert res["best"] in [r[0] for r in res["results"]]
    assert torch.equal(batch.cons, before)
    assert batch.tile == res["best"][0]


@pytest.mark.parametrize("kw", [dict(riemann="LAX-FRIEDRICHS"), dict(recon_var="CONSERVATIVE"),
                                dict(interpolation_limiter=True), dict(gravity=(0.0, -1.0, 0.0)),
                                dict(nh=4, viscous=True, mu=0.01)])
def test_batch_rejects_setups_it_does_not_build(kw):
    """Checked on the host before anything touches a device."""
    from jaxfluids_gb300 import BatchedRK3
    with pytest.raises(NotImplementedError):
        BatchedRK3(_configs([(16, 16), (24, 24)], **kw), device="cpu")
