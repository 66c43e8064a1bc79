"""The multi-rank paths on CPU, with two gloo ranks (127.0.0.1).

- The benchmark's process-group setup, barrier, max-over-ranks timing,
  per-rank particle seeds and whole-job weak-scaling rate.  The E-step
  shards over particles with no exchange, so its only collectives are the
  barrier around the timed region and the max of the ranks' times.
- The insertion's exchange (tg3.dist.allreduce_insertion): two ranks each
  insert half of the particles (the oracle's insertion stands in for the
  GPU's on these CPU ranks) and sum F, T, O3D and the counter; the result
  equals one rank inserting all of them (FSC >= 0.999 and to rounding).
  This path has not run on more than one GPU: every run here has one."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK="0",
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    r, w, local = bench.init_dist()
    assert (r, w, local) == (rank, world, 0)
    bench.barrier(w)
    # ranks finish their steps at different times; the slowest sets the job's time
    ms = bench.reduce_max(w, 10.0 + 5.0 * rank)
    rate = bench.job_rate(64 * 3, ms, w)
    out.put((rank, ms, rate, bench.rank_seed(1001, r)))
    bench.barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_single_rank_helpers_need_no_process_group():
    import bench
    assert bench.reduce_max(1, 3.5) == 3.5
    bench.barrier(1)
    assert bench.rank_seed(1001, 0) == 1001
    assert bench.job_rate(128 * 150, 2000.0, 1) == pytest.approx(9600.0)


def test_two_gloo_ranks_aggregate_weak_scaling():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    for p in procs:
        if p.is_alive():
            p.kill()
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    (_, ms0, v0, s0), (_, ms1, v1, s1) = res
    assert ms0 == ms1 == 15.0                      # max over ranks, on every rank
    assert v0 == v1 == pytest.approx(64 * 3 * 2 / 0.015)
    assert s0 != s1                                # each rank has its own particles


def _insert_rank(rank, world, port, out, case):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK="0",
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "thunder-refactor-expectation_gb300"))
    import numpy as np
    import torch
    import torch.distributed as dist
    from tg3 import dist as tdist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    F, T, O3, n = _oracle_insert(case, range(rank, case["n"], world))
    Ft = torch.as_tensor(F)
    Tt = torch.as_tensor(T)
    Ot = torch.as_tensor(O3)
    ct = torch.tensor([n], dtype=torch.int64)
    tdist.allreduce_insertion(Ft, Tt, Ot, ct)
    if rank == 0:
        out.put((Ft.numpy(), Tt.numpy(), Ot.numpy(), int(ct.item())))
    dist.barrier()
    dist.destroy_process_group()


def _insert_case(kernel):
    import numpy as np
    sys.path.insert(0, str(ROOT / "thunder-refactor-expectation_gb300"))
    from tg3 import synth
    rng = np.random.default_rng(31)
    box, pf, px, rU, n = 32, 2, 1.5, 10, 24
    bm = synth.blob_map(rng, 20, (2.0, 4.0), px, 9.0)
    st = synth.make_stack(32, [bm], box, px, pf, rU, synth.config_rL(box, px), n, 2.0, 1.0)
    return dict(n=n, box=box, pf=pf, kernel=kernel, dat=st.dat, ctf=st.ctf, iCol=st.iCol,
                iRow=st.iRow, quat=st.quat_true, trans=st.trans_true,
                off=rng.uniform(-0.5, 0.5, (n, 2)), w=rng.random(n) + 0.5)


def _oracle_insert(c, images):
    import numpy as np
    from oracle import oracle as O
    vd = c["pf"] * c["box"]
    F = np.zeros((vd, vd, vd // 2 + 1), np.complex128)
    T = np.zeros(F.shape)
    O3 = np.zeros(3)
    n = 0
    b = (c["pf"] * 1.9) ** 2
    tab = O.mkb_table(1.9, 15.0, b, 100000)
    mats = O.rotmat(c["quat"])
    for l in images:
        tt = c["trans"][l] - c["off"][l]
        img = O.translate_image(c["dat"][l], -tt[0], -tt[1], c["box"], c["iCol"], c["iRow"])
        O.insert(F, T, img, c["ctf"][l], mats[l], float(c["w"][l]), c["iCol"] * c["pf"],
                 c["iRow"] * c["pf"], c["kernel"], c["pf"] * 1.9, tab, b)
        O3 -= mats[l].reshape(3, 3)[:, :2] @ tt
        n += 1
    return F, T, O3, n


@pytest.mark.parametrize("kernel", [0, 1])
def test_two_gloo_ranks_sum_their_insertions(kernel):
    import numpy as np
    from oracle import oracle as O
    mp = pytest.importorskip("torch.multiprocessing")
    case = _insert_case(kernel)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_insert_rank, args=(r, 2, port, q, case)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        if p.is_alive():
            p.kill()
        assert p.exitcode == 0
    F2, T2, O2, n2 = res
    F1, T1, O1, n1 = _oracle_insert(case, range(case["n"]))
    assert n2 == n1 == case["n"]
    assert np.abs(F2 - F1).max() < 1e-12 * np.abs(F1).max()
    assert np.abs(T2 - T1).max() < 1e-12 * np.abs(T1).max()
    np.testing.assert_allclose(O2, O1, rtol=0, atol=1e-12)
    # FSC over the shells the particles reach (pf x cutoff 10)
    fsc = O.fsc(F2, F1, case["pf"] * 10)
    assert fsc[1:].min() >= 0.999
