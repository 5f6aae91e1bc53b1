"""Basis-pruning network kernels on the GPU: the tcgen05 BF16 GEMM against exact integer
products, and (below) the forward/backward passes against the NumPy oracle."""

import numpy as np
import pytest
import torch

from impuritymodel_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _ptr(t):
    return t.data_ptr()


# The tile width is the widest of 256, 64 and 16 columns dividing N that still gives four
# fifths of the SMs a tile: with 152 SMs, (19456, 256, 64) runs 256-column tiles, (4096, 256,
# 320) and (4096, 320, 128) 64-column tiles, the small shapes 16-column tiles; K = 64 is one K
# tile, K = 320 more tiles than the ring has stages.
@pytest.mark.parametrize("M,N,K,offset", [(128, 256, 64, 0), (256, 64, 320, 0), (384, 48, 128, 0),
                                          (128, 16, 64, 0), (256, 320, 256, 0), (19456, 256, 64, 0),
                                          (4096, 256, 320, 0), (4096, 320, 128, 0), (256, 64, 1024, 1)])
def test_gemm_bf16_exact(eng, M, N, K, offset):
    """Small integers are exact in BF16 and their products' sums exact in FP32, so the tensor
    core result must equal the integer product bit for bit (checks the bulk-tensor copies,
    operand layouts, descriptors, the stage ring and the accumulator read-back).  ``offset``
    shifts C by one float off 16-byte alignment (the epilogue's element-wise stores)."""
    rng = np.random.default_rng(M + N + K)
    a = rng.integers(-4, 5, size=(M, K)).astype(np.float32)
    b = rng.integers(-4, 5, size=(N, K)).astype(np.float32)
    A = torch.from_numpy(a).to(eng.device).to(torch.bfloat16).contiguous()
    B = torch.from_numpy(b).to(eng.device).to(torch.bfloat16).contiguous()
    Cbuf = torch.full((M * N + offset,), np.nan, dtype=torch.float32, device=eng.device)
    C = Cbuf[offset:].view(M, N)
    eng.reset_status()
    L.check(eng.lib.edgpu_gemm_bf16(_ptr(A), _ptr(B), M, N, K, _ptr(C), _ptr(eng.status), eng.stream), "gemm")
    eng.read_status("gemm")
    assert np.array_equal(C.cpu().numpy(), a @ b.T)


def _rand_states(rng, B, n_orb, n_el, words=5):
    w = np.zeros((B, words), dtype=np.uint64)
    for b in range(B):
        for i in rng.choice(n_orb, n_el, replace=False):
            w[b, i // 64] |= np.uint64(1) << np.uint64(63 - i % 64)
    return w


@pytest.mark.parametrize("B", [256, 4096])
def test_mlp_gradients_match_oracle(eng, B):
    """Forward output and every gradient of one batch against the CPU oracle (same BF16
    rounding points, float64 sums): relative Frobenius error < 1e-2 (the device accumulates in
    FP32, and an FP32/float64 difference can flip a BF16 rounding of one activation).  Batch
    256 runs every GEMM on 16-column tiles; batch 4096 runs the forward and the ReLU-mask
    GEMMs on 64-column tiles."""
    from oracle import mlp_oracle as MO
    from impuritymodel_gb300 import pruning

    rng = np.random.default_rng(5)
    net = pruning.BasisNet(eng, seed=3)
    with torch.no_grad():
        for k in ("b1", "b2"):
            net.p[k].copy_(torch.from_numpy(rng.normal(size=net.p[k].shape[0]) * 0.1).float())
    net.refresh()
    w = _rand_states(rng, B, 316, 60)
    st = torch.from_numpy(w.view(np.int64)).to(eng.device)
    target = torch.from_numpy(rng.normal(size=B) - 7.0).float().to(eng.device)
    X, Xt = net.inputs(st, transposed=True)
    Xh = MO.bits(w, pruning.N_IN)
    assert np.array_equal(X.float().cpu().numpy(), Xh)
    assert np.array_equal(Xt.float().cpu().numpy(), Xh.T)
    eng.reset_status()
    loss = net.gradients(X, Xt, target)
    eng.read_status("mlp gradients")
    p = {k: v.double().cpu().numpy() for k, v in net.p.items()}
    y_ref, _ = MO.forward(Xh, p)
    y, _ = net.forward(X)
    assert np.abs(y.double().cpu().numpy() - y_ref).max() < 1e-2 * np.abs(y_ref).max()
    loss_ref, g_ref = MO.grads(Xh, target.double().cpu().numpy(), p)
    assert abs(float(loss) - loss_ref) < 1e-3 * loss_ref
    for k, gr in g_ref.items():
        gd = net.g[k].double().cpu().numpy()
        assert np.linalg.norm(gd - gr) <= 1e-2 * np.linalg.norm(gr) + 1e-12, k


def test_mlp_forward_wide_tiles(eng):
    """Forward pass of a batch of 19456 states (152 row tiles: the bias + ReLU GEMMs run on
    256-column tiles) against the CPU oracle."""
    from oracle import mlp_oracle as MO
    from impuritymodel_gb300 import pruning

    rng = np.random.default_rng(9)
    net = pruning.BasisNet(eng, seed=4)
    with torch.no_grad():
        for k in ("b1", "b2"):
            net.p[k].copy_(torch.from_numpy(rng.normal(size=net.p[k].shape[0]) * 0.1).float())
    net.refresh()
    B = 19456
    w = _rand_states(rng, B, 316, 60)
    st = torch.from_numpy(w.view(np.int64)).to(eng.device)
    X, _ = net.inputs(st, transposed=False)
    eng.reset_status()
    y, _ = net.forward(X)
    eng.read_status("mlp forward")
    p = {k: v.double().cpu().numpy() for k, v in net.p.items()}
    y_ref, _ = MO.forward(MO.bits(w, pruning.N_IN), p)
    assert np.abs(y.double().cpu().numpy() - y_ref).max() < 1e-2 * np.abs(y_ref).max()


def test_trained_network_prunes_better_than_random(eng):
    """Trained on the ground states of 40 seeded models (10-30 bath spin-orbitals), the network
    ranks the basis of a held-out model.  Keeping the best-ranked half costs at most 1e-4 eV of
    ground-state energy, less than keeping the half with the lowest diagonal energies (the
    ranking without the network) or a random half."""
    from impuritymodel_gb300 import models as M
    from impuritymodel_gb300 import pruning

    train = [M.random_model(1000 + s, 1 + s % 3) for s in range(40)]
    st, lw = pruning.ground_state_samples(eng, train)
    net = pruning.BasisNet(eng, seed=0, lr=2e-3)
    log = []
    net.train(st, lw, epochs=30, batch=512, log=log)
    assert log[-1] < 0.8 * log[0], log
    held = M.random_model(2000, 3)
    r_net = pruning.pruned_ground_state(eng, held, 0.5, net)
    r_diag = pruning.pruned_ground_state(eng, held, 0.5, "diagonal")
    r_rand = pruning.pruned_ground_state(eng, held, 0.5, "random")
    assert r_net["error"] >= -1e-9 and r_net["error"] <= 1e-4, r_net
    assert r_net["error"] < r_diag["error"] and r_net["error"] < r_rand["error"], (r_net, r_diag, r_rand)
    # the drop-in path: pruned bytes basis through finite.eigensystem
    from impuritymodel_gb300 import finite

    basis = finite.get_basis(*held.basis_args())
    kept = pruning.prune_basis(held.n_spin_orbitals, basis, net, 0.5)
    assert len(kept) == r_net["n_pruned"] and set(kept) <= set(basis)
    es, _ = finite.eigensystem(held.n_spin_orbitals, held.hOp, kept, 1)
    assert abs(es[0] - (r_net["e_full"][0] + r_net["error"])) < 1e-9
