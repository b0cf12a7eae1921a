"""Continuous-batching server (mbcg_server_*): results are the same alone and in a mix, and
match the single-case API; admission respects the arena; bookkeeping is exact.

Tolerances: a lattice served alone or in any mix runs the same batch-kernel code on the same
data, so its final state is compared bit for bit (fetched fields and the 64-bit state hash).
The single-case API runs a separately compiled kernel (which may fuse different multiply-add
pairs), so served and single-case results are each held to the parity gates against the FP64
oracle instead.
"""
import numpy as np
import pytest

import mbcg
import oracle_lib as ol
from gpu_util import assert_fp32_parity, group_errors, written_nodes

pytestmark = pytest.mark.gpu


def mix_cases():
    """Small cases of every kind the server batches: both lattices, three storage forms,
    periodic / wall / inlet-outlet boundaries."""
    out = []
    out.append((mbcg.bubble_params(30, q=19, radius=8.0, tau=0.8, sigma=0.01), 40))
    out.append((mbcg.bubble_params(34, q=27, radius=9.0, tau=0.8, sigma=0.01, precision=mbcg.FP16), 30))
    out.append((mbcg.rti_params(24, 40, q=27), 25))
    out.append((mbcg.rti_params(20, 44, q=19, precision=mbcg.FP16), 35))
    out.append((mbcg.jet_params(40, 36, 50, q=27, diameter=10.0), 20))
    out.append((mbcg.jet_params(34, 34, 40, q=19, diameter=8.0, precision=mbcg.BF16), 17))
    out.append((mbcg.bubble_params(46, q=27, radius=12.0, tau=0.7, sigma=0.005), 33))
    return out


def run_alone(cases):
    res = []
    with mbcg.Server(keep_results=1, chunk_steps=8, calibrate=0, zchunk=16) as srv:
        for p, n in cases:
            rid = srv.submit(p, n)
            info = srv.wait(rid)
            assert info.state == mbcg.REQ_DONE, info.as_dict()
            res.append((info.state_hash, srv.fetch(rid, p.shape), info.as_dict()))
            srv.release(rid)
    return res


def test_same_result_alone_and_in_the_mix():
    cases = mix_cases()
    alone = run_alone(cases)
    # the mix: few slots so that lattices are admitted while others run, staggered submission
    with mbcg.Server(keep_results=1, chunk_steps=8, calibrate=0, zchunk=16, max_live=3) as srv:
        ids = []
        for i, (p, n) in enumerate(cases):
            ids.append(srv.submit(p, n))
            if i == 2:
                srv.wait(ids[0])
        infos = [srv.wait(r) for r in ids]
        st = srv.stats()
        assert st.compositions > 2  # the batch composition changed as lattices came and went
        for (p, n), rid, info, (h0, f0, _) in zip(cases, ids, infos, alone):
            assert info.state == mbcg.REQ_DONE and info.status == 0
            assert info.steps_done == n
            assert info.state_hash == h0
            np.testing.assert_array_equal(srv.fetch(rid, p.shape)[written_nodes(p)], f0[written_nodes(p)])
            srv.release(rid)


# 16-bit storage: colour densities by relative L2 (the storage-form bounds of the jet test);
# velocity and stress by RMS error in units of their storage scale (u_ref, pi_scale), since a
# static bubble's velocities are spurious currents far below the scale, where relative errors
# measure only the format's resolution
FORM_BOUNDS = {mbcg.FP16: {"rhor": 5e-3, "rhob": 1e-3, "u": 2e-3, "Pi": 2e-3},
               mbcg.BF16: {"rhor": 5e-2, "rhob": 1e-2, "u": 2e-2, "Pi": 2e-2}}


def form_errors(got, ref, idx, p):
    e = group_errors(got, ref, idx)
    g, r = got[idx], ref[idx]
    e["u"] = float(np.sqrt(np.mean((g[2:5].astype(np.float64) - r[2:5]) ** 2))) / p.u_ref
    e["Pi"] = float(np.sqrt(np.mean((g[5:11].astype(np.float64) - r[5:11]) ** 2))) / p.pi_scale
    return e


def test_server_and_single_case_api_match_the_oracle():
    """FP32: served results and single-case results both meet the parity gate against the FP64
    oracle run from the same initial condition (the FP32 gate: relative L2 1e-5, or 3x the
    reference's own FP32 arithmetic where that is larger); in FP16 / BF16 storage the served
    and single-case runs agree within FORM_BOUNDS."""
    cases = mix_cases()
    alone = run_alone(cases)
    for (p, n), (_, f, info) in zip(cases, alone):
        with mbcg.Case(p) as c:
            c.init()
            c.step(n)
            single = c.copy_out()
            d = c.diagnostics()
        idx = written_nodes(p)
        if p.precision == mbcg.FP32:
            a0 = ol.oracle_init(p, np.float64)
            ref64 = ol.oracle_run(p, a0.copy(), n)
            ref32 = ol.oracle_run(p, a0.astype(np.float32), n)
            assert_fp32_parity(f, ref64, ref32, idx, what=f"served {p.describe()['ic']}")
            assert_fp32_parity(single, ref64, ref32, idx, what=f"single {p.describe()['ic']}")
        else:
            # the 16-bit forms' own accuracy is the subject of tests/test_gpu_forms.py; here the
            # served and single-case runs of the same form must agree within its resolution
            e = form_errors(f, single, idx, p)
            for k, lim in FORM_BOUNDS[p.precision].items():
                assert e[k] < lim, (p.describe(), k, e)
        assert abs(info["diag"]["mass_r"] - d["mass_r"]) <= 1e-5 * abs(d["mass_r"]) + 1e-9


def test_admission_by_footprint_and_accounting():
    cases = [(mbcg.bubble_params(L, q=q, radius=L / 4, tau=0.8, sigma=0.01), n)
             for L, q, n in ((30, 19, 30), (62, 27, 20), (46, 19, 25), (38, 27, 40), (54, 19, 15))]
    big = max(4 * 2 * 11 * (p.nx + 7) // 8 * 8 * p.ny * p.nz for p, _ in cases)
    arena = int(1.3 * big) + (1 << 20)  # room for the largest lattice and little else
    with mbcg.Server(arena_bytes=arena, chunk_steps=4, calibrate=0) as srv:
        ids = [srv.submit(p, n) for p, n in cases]
        srv.drain()
        st = srv.stats()
        assert st.completed == len(cases) and st.failed == 0
        assert st.arena_peak_bytes <= st.arena_bytes
        assert st.node_updates == sum(p.active_nodes() * n for p, n in cases)
        infos = [srv.poll(r) for r in ids]
        assert all(i.state == mbcg.REQ_DONE for i in infos)
        # at most two of these fit at once: some requests waited for memory
        assert max(i.t_admit for i in infos) > min(i.t_done for i in infos)
        for i in infos:
            assert i.t_submit <= i.t_admit <= i.t_done


def test_zero_steps_and_rejections():
    with mbcg.Server(arena_bytes=64 << 20, calibrate=0, keep_results=1) as srv:
        p = mbcg.bubble_params(30, q=19, radius=8.0)
        rid = srv.submit(p, 0)
        info = srv.wait(rid)
        assert info.state == mbcg.REQ_DONE and info.steps_done == 0
        with mbcg.Case(p) as c:
            c.init()
            ref = c.copy_out()
        np.testing.assert_array_equal(srv.fetch(rid, p.shape)[written_nodes(p)], ref[written_nodes(p)])
        srv.release(rid)
        with pytest.raises(mbcg.MbcgError):
            srv.submit(mbcg.bubble_params(200, q=27), 10)  # larger than the arena


def test_calibrated_cost_model_and_planner():
    with mbcg.Server(arena_bytes=4 << 30, calibrate=1, keep_results=1) as srv:
        st = srv.stats().as_dict()
        ns = st["plane_ns"]
        assert all(v > 0 for v in ns.values())
        # D3Q27 costs more per plane than D3Q19 in the same storage
        assert ns["q27_f32"] > ns["q19_f32"] and ns["q27_f32_periodic"] > ns["q19_f32_periodic"]
        assert 0.0 <= st["tile_overhead_planes"] <= 32.0
        p = mbcg.bubble_params(40, q=27, radius=10.0)
        rid = srv.submit(p, 12)
        info = srv.wait(rid)
        assert info.state == mbcg.REQ_DONE
        assert srv.stats().zchunk in (8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256, 512)
        got = srv.fetch(rid, p.shape)
    # the planner's depth never changes the result
    with mbcg.Server(calibrate=0, zchunk=5, keep_results=1) as srv:
        rid = srv.submit(p, 12)
        assert srv.wait(rid).state == mbcg.REQ_DONE
        np.testing.assert_array_equal(srv.fetch(rid, p.shape)[written_nodes(p)], got[written_nodes(p)])
