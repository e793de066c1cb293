"""The N > 1 host path of bench.py on the CPU: two gloo ranks, as torchrun
starts them, combine their figures the way a multi-GPU run does (the
slowest rank's time, the units of all ranks), and the reference arm runs on
rank 0 only.  No GPU and no collective on the data path: the ranks are
independent replicas."""
import contextlib
import io
import os
import socket
import types

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench

    pg = bench.init_replicas(world)
    try:
        ms = bench.max_over_ranks(pg, [3.0, 5.0][rank])
        units = bench.sum_over_ranks(pg, [100_000, 250_000][rank])
        # an end-to-end loop each rank timed on its own (seconds per step)
        e2e = bench.replica_rate(pg, [1_000_000, 1_000_000][rank], [0.002, 0.004][rank])
        pg.barrier()
        printed = ""
        if rank == 1:  # the reference arm stands down off rank 0, before any work
            buf = io.StringIO()
            with contextlib.redirect_stdout(buf):
                bench.run_reference(types.SimpleNamespace(n=10, steps=1, warmup=1, gpus=world))
            printed = buf.getvalue()
        out.put((rank, ms, units, bench.job_rate(units, ms), e2e, printed))
    finally:
        pg.destroy_process_group()


def test_two_gloo_replicas_combine_like_torchrun():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, units, rate, e2e, printed in results:
        assert ms == 5.0  # the slowest rank's time
        assert units == 350_000  # every rank's units
        assert rate == pytest.approx(350_000 / 5e-3 / 1e6)
        assert e2e == pytest.approx(2_000_000 / 0.004 / 1e6)  # both ranks' points over the slower loop
        assert printed == ""


def test_single_process_needs_no_group():
    import bench

    assert bench.init_replicas(1) is None
    assert bench.max_over_ranks(None, 2.5) == 2.5
    assert bench.sum_over_ranks(None, 7) == 7
    assert bench.job_rate(10_000_000, 0.8) == pytest.approx(12_500.0)
    assert bench.replica_rate(None, 10_000_000, 0.002) == pytest.approx(5_000.0)
