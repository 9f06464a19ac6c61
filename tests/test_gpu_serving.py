"""Serving engine (cyr_server_*): every request gives the same result in the mix
as alone through cyr_cuda_main, within the parity tolerance, with identical
NaN masks; admission by footprint, graph capture/replay and device buffers.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cyrsoxs_gb300 import _native, serving

    return torch, _native, serving


def options_for(nat, case, **over):
    kv = [[0.0, 0.0, 1.0]] if case.case_type == 0 else [cases._normalize32(k).tolist() for k in case.kvecs]
    kw = dict(nx=case.nx, ny=case.ny, nz=case.nz, num_material=case.num_material, energies=case.energies,
              start_angle=case.angles[0], end_angle=case.angles[1], increment_angle=case.angles[2],
              phys_size=case.phys_size, case_type=case.case_type, k_vectors=kv, detector=case.detector,
              morphology_type=case.morphology, ewald_interpolation=case.interpolation, windowing=case.windowing,
              scatter_approach=case.scatter, algorithm=case.algorithm, max_streams=case.max_streams,
              rot_mask=case.rot_mask, reference_frame=case.frame)
    kw.update(over)
    return nat.Options(**kw)


def same(got, want):
    assert got.shape == want.shape
    assert np.array_equal(np.isnan(got), np.isnan(want)), "NaN masks differ"
    ok = ~np.isnan(want)
    g, w = got[ok].astype(np.float64), want[ok].astype(np.float64)
    peak = np.abs(w).max()
    sel = np.abs(w) > 1e-6 * peak
    assert (np.abs(g[sel] - w[sel]) / np.abs(w[sel])).max() <= TOL


# a mix of shapes, morphologies, frames, interpolation, strategies and sizes
MIX = ["euler_sphere", "vector_nn_full", "euler_hanning_mask", "material_frame", "beam_divergence", "grazing", "twod",
       "odd_sizes", "alg1_streams", "four_materials", "nonsquare", "c1_slice"]


# a size with prime factors above 7 on every axis (Bluestein transforms)
EXTRA = {"prime_mix": cases.Case("prime_mix", 37, 29, 11, 2, [283.0, 287.0], seed=61, geometry="blobs",
                                 angles=(0.0, 150.0, 30.0))}


def mix_requests(nat):
    reqs = []
    for i, n in enumerate(MIX + list(EXTRA)):
        c = EXTRA[n] if n in EXTRA else cases.CASES[n]
        strategy = (0, 1, 2)[i % 3]
        reqs.append((n, options_for(nat, c, strategy=strategy), cases.optical_constants(c),
                     np.ascontiguousarray(cases.voxels(c), np.float32), c))
    return reqs


def out_for(nat, opts, c):
    s = opts.struct
    return np.zeros((s.num_energies, opts.num_k, s.ny, s.nx), np.float32)


def test_each_request_is_the_same_alone_and_in_the_mix():
    torch, nat, serving = _setup()
    reqs = mix_requests(nat)
    alone = {n: nat.cuda_main(o, opt, v, streams_variant=c.algorithm == 1) for n, o, opt, v, c in reqs}
    with serving.Server(slots=4, graphs=True) as srv:
        for rnd in range(3):  # repeats: warm runs, graph captures, replays
            outs, ids = {}, {}
            for n, o, opt, v, c in reqs:
                outs[n] = out_for(nat, o, c)
                ids[n] = srv.submit(o, opt, v, outs[n])
            for n in ids:
                lat, q = srv.wait(ids[n])
                assert lat >= q >= 0.0
                same(outs[n], alone[n])
        st = srv.stats()
    assert st["completed"] == 3 * len(reqs) and st["failed"] == 0


def test_one_slot_captures_then_replays_a_repeated_signature():
    torch, nat, serving = _setup()
    n, o, opt, v, c = mix_requests(nat)[1]
    want = nat.cuda_main(o, opt, v)
    with serving.Server(slots=1, graphs=True) as srv:
        for _ in range(4):
            out = out_for(nat, o, c)
            srv.wait(srv.submit(o, opt, v, out))
            same(out, want)
        st = srv.stats()
    assert st["graph_captures"] == 1 and st["graph_replays"] == 2


def test_budget_smaller_than_a_request_still_runs_requests_one_at_a_time():
    torch, nat, serving = _setup()
    reqs = mix_requests(nat)[:4]
    with serving.Server(slots=4, hbm_budget=1) as srv:
        outs = [out_for(nat, o, c) for _, o, _, _, c in reqs]
        ids = [srv.submit(o, opt, v, out) for (_, o, opt, v, _), out in zip(reqs, outs)]
        for (n, o, opt, v, c), out, rid in zip(reqs, outs, ids):
            srv.wait(rid)
            same(out, nat.cuda_main(o, opt, v, streams_variant=c.algorithm == 1))


def test_device_buffers():
    torch, nat, serving = _setup()
    n, o, opt, v, c = mix_requests(nat)[0]
    want = nat.cuda_main(o, opt, v)
    dv = torch.from_numpy(v).cuda()
    dout = torch.zeros(want.size, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    with serving.Server(slots=2) as srv:
        srv.wait(srv.submit(o, opt, dv.data_ptr(), dout.data_ptr(), device=True))
    same(dout.cpu().numpy().reshape(want.shape), want)


def test_invalid_request_is_rejected_at_submit():
    torch, nat, serving = _setup()
    bad = nat.Options(nx=4099, ny=2, nz=1, num_material=1, energies=[285.0], start_angle=0, end_angle=0,
                      increment_angle=0, phys_size=5.0)  # prime, beyond the Bluestein limit
    with serving.Server(slots=1) as srv:
        with pytest.raises(nat.CyrError):
            srv.submit(bad, np.zeros((1, 1, 4), np.float32), np.zeros((1, 1, 2, 4099, 4), np.float32),
                       np.zeros((1, 1, 2, 4099), np.float32))


def test_one_slot_alternating_signatures_after_a_capture():
    # A runs warm, is captured, then B runs uncaptured on the same slot after A's graph, and so on
    torch, nat, serving = _setup()
    reqs = mix_requests(nat)
    a, b = reqs[1], reqs[2]
    want = {r[0]: nat.cuda_main(r[1], r[2], r[3]) for r in (a, b)}
    with serving.Server(slots=1, graphs=True) as srv:
        for r in (a, a, b, a, b, b, a):
            n, o, opt, v, c = r
            out = out_for(nat, o, c)
            srv.wait(srv.submit(o, opt, v, out))
            same(out, want[n])
        st = srv.stats()
    # B's first run may grow the slot's buffers, which retires A's graph (it is captured again later)
    assert st["failed"] == 0 and st["graph_captures"] >= 2 and st["graph_replays"] >= 1


# Request groups (CYR_SERVER_GROUPS): same-shape FIELDS requests on device buffers, queued behind a
# running request, share one launch per kernel; each must equal its own cuda_main result.
GROUP_SHAPES = [
    # (nx, nz, materials, energies, windowing, rot_mask): warp-FFT rows (fused build) and 40-point rows
    (64, 16, 2, [281.0, 284.0, 285.5, 289.0], 0, 0),
    (128, 32, 3, [283.0, 286.0, 287.0], 1, 1),
    (40, 8, 2, [284.0, 286.0], 0, 0),
]


@pytest.mark.parametrize("shape", GROUP_SHAPES, ids=lambda s: f"{s[0]}x{s[0]}x{s[1]}m{s[2]}")
def test_grouped_requests_equal_their_single_results(shape):
    torch, nat, serving = _setup()
    nx, nz, m, es, win, mask = shape
    members = []
    for i in range(6):
        c = cases.Case(f"grp{i}", nx, nx, nz, m, [e + 0.5 * i for e in es], seed=90 + i, geometry="blobs",
                       windowing=win, rot_mask=mask, angles=(0.0, 150.0, 30.0))
        o = options_for(nat, c, strategy=2)
        opt, v = cases.optical_constants(c), np.ascontiguousarray(cases.voxels(c), np.float32)
        members.append((o, opt, torch.from_numpy(v).cuda(), nat.cuda_main(o, opt, v), c))
    outs = [torch.zeros(w.size, dtype=torch.float32, device="cuda") for _, _, _, w, _ in members]
    torch.cuda.synchronize()
    with serving.Server(slots=1, groups=True) as srv:
        # the first request occupies the only slot, so the other five queue and are admitted as one group
        ids = [srv.submit(o, opt, dv.data_ptr(), out.data_ptr(), device=True)
               for (o, opt, dv, _, _), out in zip(members, outs)]
        for rid in ids:
            srv.wait(rid)
        st = srv.stats()
    assert st["group_runs"] >= 1 and st["grouped_requests"] >= 2, st
    for (o, opt, dv, want, c), out in zip(members, outs):
        same(out.cpu().numpy().reshape(want.shape), want)


def test_groups_and_graphs_mix_with_other_requests():
    torch, nat, serving = _setup()
    reqs = mix_requests(nat)
    alone = {n: nat.cuda_main(o, opt, v, streams_variant=c.algorithm == 1) for n, o, opt, v, c in reqs}
    dev = {n: torch.from_numpy(v).cuda() for n, o, opt, v, c in reqs}
    with serving.Server(slots=2, graphs=True, groups=True) as srv:
        for rnd in range(2):
            outs, ids = {}, {}
            for n, o, opt, v, c in reqs + reqs:  # each request twice: same-key pairs can group
                key = (n, len(ids))
                outs[key] = torch.zeros(alone[n].size, dtype=torch.float32, device="cuda")
                ids[key] = srv.submit(o, opt, dev[n].data_ptr(), outs[key].data_ptr(), device=True)
            for key, rid in ids.items():
                srv.wait(rid)
                same(outs[key].cpu().numpy().reshape(alone[key[0]].shape), alone[key[0]])


def test_profiling_around_graph_capture_and_replay():
    # launches captured into a slot's graph (and its replays) are not timed; the profile still ends cleanly
    torch, nat, serving = _setup()
    n, o, opt, v, c = mix_requests(nat)[1]
    want = nat.cuda_main(o, opt, v)
    with serving.Server(slots=1, graphs=True) as srv:
        nat.profile_begin()
        for _ in range(3):  # warm run, capture, replay
            out = out_for(nat, o, c)
            srv.wait(srv.submit(o, opt, v, out))
            same(out, want)
        prof, dropped = nat.profile_end()
        st = srv.stats()
    assert st["graph_captures"] == 1 and st["graph_replays"] == 1
    assert dropped > 0  # the captured launches
    assert sum(v[0] for v in prof.values()) > 0  # the warm run's launches were timed
