"""The learned MIS proposal's tensor-core kernels against the CPU network oracle
(oracle/plt_oracle_mlp.cpp, same BF16 storage rounding, exact accumulation):

- forward outputs on a batch drawn from the exact samplers;
- the gradient of the mean weighted mixture NLL (the backward kernels), parameter by parameter;
- training with Adam reduces the loss on fresh batches.

Tolerances are written in the tests: the GPU accumulates in FP32 in another order, so a stored
BF16 value can round the other way now and then; the bounds are on relative L2 errors and on the
share of entries within a per-entry tolerance.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FORWARD_REL_L2 = 2e-3
GRAD_REL_L2 = 2e-2
GRAD_ENTRY_RTOL = 5e-2
GRAD_ENTRY_SHARE = 0.98


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch


@pytest.fixture(scope="module")
def ctx(torch_cuda, product_lib, profiles):
    from pltfalcor_gb300 import scene as S
    from pltfalcor_gb300.bsdf import PLTContext
    c = PLTContext()
    c.set_spectral_profiles(profiles[0])
    c.set_materials(S.small_scene().records)
    c.proposal_init(7)
    yield c
    c.close()


def _batch(ctx, n, seed):
    x, t, w = ctx.proposal_generate(n, seed)
    return x, t, w, x.cpu().numpy().view(np.uint16), t.cpu().numpy(), w.cpu().numpy()


def test_generated_batch(ctx):
    x, t, w, xb, tn, wn = _batch(ctx, 8192, 3)
    assert (wn >= 0).all() and (wn <= 4).all()
    assert 0.3 < (wn > 0).mean() <= 1.0                 # most queries give a non-delta direction
    assert ((tn >= 0) & (tn < 1)).all()                  # targets: primary samples in [0,1)^2
    # uniform primary samples: their mean is near the centre of the square
    assert np.abs(tn.mean(0) - 0.5).max() < 0.02
    onehot = xb[:, 6:14].view(np.uint16)
    assert ((onehot == 0x3F80).sum(1) == 1).all()        # exactly one class bit (bf16 1.0)


def test_forward_matches_oracle(ctx, oracle_lib):
    import oracle
    x, t, w, xb, tn, wn = _batch(ctx, 4096, 5)
    g = ctx.proposal_forward(x).cpu().numpy()
    o = oracle.mlp_forward(ctx.proposal_params(), xb)
    err = np.linalg.norm(g - o) / np.linalg.norm(o)
    assert err < FORWARD_REL_L2, err


def test_gradient_matches_oracle(ctx, oracle_lib):
    import oracle
    x, t, w, xb, tn, wn = _batch(ctx, 4096, 11)
    loss, g = ctx.proposal_gradient(x, t, w)
    g = g.cpu().numpy().astype(np.float64)
    oloss, og = oracle.mlp_gradient(ctx.proposal_params(), tn, wn, x_bits=xb)
    assert abs(loss - oloss) <= 1e-3 * abs(oloss) + 1e-5, (loss, oloss)
    rel = np.linalg.norm(g - og) / np.linalg.norm(og)
    scale = np.abs(og).max()
    ok = np.abs(g - og) <= GRAD_ENTRY_RTOL * np.maximum(np.abs(og), 1e-3 * scale)
    print("gradient rel L2 %.3g, entries within %.0e: %.4f" % (rel, GRAD_ENTRY_RTOL, ok.mean()))
    assert rel < GRAD_REL_L2, rel
    assert ok.mean() >= GRAD_ENTRY_SHARE, ok.mean()
    # per layer: every weight block gets a non-zero gradient
    for lo, hi in ((0, 1024), (1024, 5120), (5120, 9216), (9216, 11264)):
        assert np.abs(g[lo:hi]).max() > 0


def test_training_reduces_loss(ctx):
    hist = ctx.proposal_train(40, batch=16384, lr=1e-3, seed=3)
    assert np.isfinite(hist).all()
    first, last = hist[:5].mean(), hist[-5:].mean()
    print("loss %.4f -> %.4f" % (first, last))
    assert last < first - 0.05 * abs(first), (first, last)
    p = ctx.proposal_params()
    assert np.isfinite(p).all()


def test_data_parallel_training_single_rank(torch_cuda, product_lib, profiles):
    """The host-side data-parallel loop (pltfalcor_gb300.distributed) with one gloo rank: library
    gradient, rank average, library Adam step; the loss falls as with plt_proposal_train."""
    import socket
    import torch.distributed as dist
    from pltfalcor_gb300 import distributed as D
    from pltfalcor_gb300 import scene as S
    from pltfalcor_gb300.bsdf import PLTContext
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=0, world_size=1)
    try:
        c = PLTContext()
        c.set_spectral_profiles(profiles[0])
        c.set_materials(S.small_scene().records)
        c.proposal_init(9)
        hist = D.train_proposal_data_parallel(c, 40, 16384, 1e-3, 3, dist)
        c.close()
    finally:
        dist.destroy_process_group()
    assert np.isfinite(hist).all()
    assert hist[-5:].mean() < hist[:5].mean() - 0.05 * abs(hist[:5].mean())
