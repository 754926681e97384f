"""The multi-rank layout on CPU with two gloo ranks (file rendezvous).  Cells are independent within a
step, so ranks that each run their own y-slab (with its halo rows) reproduce a
single-process run over the whole block; the only collective is the max of the
ranks' timers, as in bench.py under torchrun."""
import os
import time

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from uclales_salsa_gb300.inputs import make_inputs, make_outputs

Y = 6            # interior y rows, split 3 + 3


def _case():
    return make_inputs("grid256x256x128", "cpu", X=4, Y=Y, Z=4)


def _slab(t, y0, y1):
    """Rows y0..y1-1 of the interior with two halo rows on each side (y is dim -3)."""
    return t[..., y0:y1 + 4, :, :].contiguous()


def _rank(rank, world, store, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from oracle_ref import Oracle
    # a file rendezvous: no port to pick, so no race with other processes for one
    dist.init_process_group("gloo", init_method="file://" + store, rank=rank, world_size=world)
    inp = _case()
    y0, y1 = rank * (Y // world), (rank + 1) * (Y // world)
    inp.fields = {k: _slab(v, y0, y1) for k, v in inp.fields.items()}
    inp.nyp = (y1 - y0) + 4
    out = make_outputs(inp)
    f = {k: v.clone() for k, v in inp.fields.items()}
    t0 = time.perf_counter()
    rc, _ = Oracle(inp.cfg).run(inp, f, out, time=1.0, nthreads=1)
    t = torch.tensor([time.perf_counter() - t0])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)       # the slowest rank's time
    # numpy arrays travel by value: a torch tensor would travel as a file descriptor that
    # this process must still serve when the parent unpickles it
    q.put((rank, rc, float(t), {k: v[..., 2:-2, :, :].numpy().copy() for k, v in out.items() if k != "diag"}))
    dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_the_single_run(tmp_path):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from oracle_ref import Oracle
    inp = _case()
    out = make_outputs(inp)
    f = {k: v.clone() for k, v in inp.fields.items()}
    rc, _ = Oracle(inp.cfg).run(inp, f, out, time=1.0, nthreads=1)
    assert rc == 0
    store = str(tmp_path / "rendezvous")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, store, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(r[1] == 0 for r in res)
    assert res[0][2] == res[1][2] > 0                # both ranks hold the max
    for k, full in out.items():
        if k == "diag":
            continue
        both = torch.cat([torch.from_numpy(res[0][3][k]), torch.from_numpy(res[1][3][k])], dim=-3)
        assert torch.equal(both, full[..., 2:-2, :, :]), k
