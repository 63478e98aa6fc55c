"""custen_compute_group: several independent handles computed by one call, free to overlap on the GPU.

The group's results must equal the same handles computed one after another, bit for bit, whether the call
runs directly or is captured into a CUDA graph and replayed; the oracle pins the values."""
import numpy as np
import pytest

import custen_gb300 as cs
import oracle
from custen_gb300.inputs import field, sentinel, sweep_operators

pytestmark = pytest.mark.gpu

N = 256


def _handles(torch, dev, inp, outs):
    hs, keep = [], []
    for (nm, v, H, L, R, V, T, B, w, fun, _), o in zip(sweep_operators(N), outs):
        wt = torch.tensor(w, device=dev, dtype=torch.float64)
        keep.append(wt)
        hs.append(cs.Stencil(v, N, N, o, inp, wt, H=H, L=L, R=R, V=V, T=T, B=B, num_tiles=2, ncoef=len(w),
                             func=cs.builtin_function(fun) if fun >= 0 else None))
    return hs, keep


def _oracle_outputs():
    inp = field(N, N, 1)
    refs = []
    for nm, v, H, L, R, V, T, B, w, fun, _ in sweep_operators(N):
        ref = sentinel(N, N)
        oracle.stencil(v, ref, inp, np.asarray(w), num_tiles=2, block_x=32, block_y=8, H=H, L=L, R=R, V=V, T=T,
                       B=B, fun_id=fun)
        refs.append(ref)
    return refs


@pytest.mark.parametrize("captured", [False, True], ids=["direct", "graph"])
def test_group_equals_one_by_one(gpu, captured):
    import torch
    dev = torch.device("cuda", 0)
    inp = torch.tensor(field(N, N, 1), device=dev)
    pre = torch.tensor(sentinel(N, N), device=dev)
    outs = [pre.clone() for _ in range(12)]
    hs, keep = _handles(torch, dev, inp, outs)
    for h in hs:      # the first Compute picks each handle's configuration (not capturable)
        h.compute()
    torch.cuda.synchronize(dev)
    for o in outs:
        o.copy_(pre)
    torch.cuda.synchronize(dev)
    s = torch.cuda.Stream(dev)
    if captured:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
            cs.compute_group(hs, cs.DEVICE, torch.cuda.current_stream(dev))
        g.replay()
    else:
        with torch.cuda.stream(s):
            cs.compute_group(hs, cs.DEVICE, s)
    s.synchronize()
    got = [o.cpu().numpy() for o in outs]
    for h in hs:
        h.destroy()
    for k, (a, r) in enumerate(zip(got, _oracle_outputs())):
        assert a.tobytes() == r.tobytes(), sweep_operators(N)[k][0]
    assert cs.device_error() == 0


def test_group_orders_against_the_callers_stream(gpu):
    """Work queued on the caller's stream before the group is seen by it; work queued after it sees the
    group's outputs."""
    import torch
    dev = torch.device("cuda", 0)
    s = torch.cuda.Stream(dev)
    inp = torch.zeros((N, N), device=dev, dtype=torch.float64)
    pre = torch.tensor(sentinel(N, N), device=dev)
    outs = [pre.clone() for _ in range(12)]
    hs, keep = _handles(torch, dev, inp, outs)
    for h in hs:
        h.compute()
    for o in outs:
        o.copy_(pre)
    src = torch.tensor(field(N, N, 1), device=dev)
    torch.cuda.synchronize(dev)
    with torch.cuda.stream(s):
        inp.copy_(src)                                  # before the group, on the caller's stream
        cs.compute_group(hs, cs.DEVICE, s)
        total = torch.stack([o.sum() for o in outs])    # after the group, on the caller's stream
    s.synchronize()
    for h in hs:
        h.destroy()
    refs = _oracle_outputs()
    for k, (o, r) in enumerate(zip(outs, refs)):
        assert o.cpu().numpy().tobytes() == r.tobytes()
    assert torch.allclose(total.cpu(), torch.tensor([r.sum() for r in refs]), rtol=1e-12, atol=1e-6)


def test_group_rejects_a_repeated_handle(gpu):
    import torch
    dev = torch.device("cuda", 0)
    inp = torch.zeros((N, N), device=dev, dtype=torch.float64)
    outs = [torch.zeros((N, N), device=dev, dtype=torch.float64) for _ in range(12)]
    hs, keep = _handles(torch, dev, inp, outs)
    with pytest.raises(cs.CustenError, match="appears twice"):
        cs.compute_group([hs[0], hs[1], hs[0]])
    for h in hs:
        h.destroy()
