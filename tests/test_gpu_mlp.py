"""GPU tests of the learned Newton start value: the tcgen05 BF16 GEMM
against torch.matmul, the device gradients and forward pass against the
float64 restatement in oracle/mlp.py (operands rounded to bfloat16 where the
device rounds them), Adam's first step, and a short training run whose
learned start value must cut the exact solver's Newton iterations."""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads
from oracle import mlp

pytestmark = pytest.mark.gpu


def _bf16(torch, shape, seed, scale=1.0):
    g = torch.Generator().manual_seed(seed)
    return (torch.randn(*shape, generator=g) * scale).to(torch.bfloat16).cuda()


@pytest.mark.parametrize("M,N,K,splits", [(128, 64, 64, 1), (300, 64, 64, 1),
                                          (1000, 16, 16, 1), (77, 32, 192, 1),
                                          (128, 64, 4096, 16), (128, 16, 8192, 32)])
def test_tc_gemm_matches_matmul(fvs, torch_cuda, M, N, K, splits):
    torch = torch_cuda
    A = _bf16(torch, (M, K), 1)
    B = _bf16(torch, (N, K), 2)
    C = torch.zeros(M, N, dtype=torch.float32, device="cuda")
    fvs.tc_gemm_bf16(A, B, C, M, N, K, splits=splits, accumulate=splits > 1)
    torch.cuda.synchronize()
    ref = A.double() @ B.double().T
    bound = (A.double().abs() @ B.double().abs().T) * 1e-5 + 1e-6
    err = (C.double() - ref).abs()
    assert bool((err <= bound).all()), float((err / bound).max())


def test_tc_gemm_strided_and_accumulating(fvs, torch_cuda):
    torch = torch_cuda
    A = _bf16(torch, (256, 96), 3)
    B = _bf16(torch, (64, 96), 4)
    C = torch.ones(256, 80, dtype=torch.float32, device="cuda")
    # K = 64 of the 96 columns, C with leading dimension 80
    fvs.tc_gemm_bf16(A, B, C, 256, 64, 64, lda=96, ldb=96, ldc=80, accumulate=True)
    torch.cuda.synchronize()
    ref = 1.0 + A[:, :64].double() @ B[:, :64].double().T
    torch.testing.assert_close(C[:, :64].double(), ref, rtol=1e-5, atol=1e-4)
    assert bool((C[:, 64:] == 1.0).all())


def test_tc_gemm_rejects_bad_shapes(fvs, torch_cuda):
    torch = torch_cuda
    A = _bf16(torch, (128, 64), 5)
    C = torch.zeros(128, 64, dtype=torch.float32, device="cuda")
    with pytest.raises(fvs.FvsError):
        fvs.tc_gemm_bf16(A, A, C, 128, 48, 64)
    with pytest.raises(fvs.FvsError):
        fvs.tc_gemm_bf16(A, A, C, 128, 64, 40)


def _problem_set(fvs, torch, n, seed, tol=1e-12):
    arr = workloads.riemann_samples(n, seed=seed)
    dev = [torch.from_numpy(a).cuda() for a in arr]
    ps = torch.empty(n, dtype=torch.float64, device="cuda")
    it = torch.empty(n, dtype=torch.int32, device="cuda")
    st = torch.empty_like(it)
    m = fvs.make_method("godunov", guess="pvrs_tr", tolerance=tol, max_iterations=200)
    fvs.exact_riemann_star(m, *dev, ps, None, it, st)
    feat = torch.empty(n, 5, dtype=torch.float32, device="cuda")
    lab = torch.empty(n, dtype=torch.float32, device="cuda")
    fvs.riemann_features(1.4, *dev, feat, pstar=ps, labels=lab)
    torch.cuda.synchronize()
    return arr, dev, feat, lab, st


def test_features_match_oracle(fvs, torch_cuda):
    arr, dev, feat, lab, st = _problem_set(fvs, torch_cuda, 4096, 11)
    ref = mlp.features(1.4, *arr)
    np.testing.assert_allclose(feat.cpu().numpy(), ref, rtol=2e-6, atol=2e-6)


def _net_with_normalization(fvs, feat, seed=7):
    net = fvs.LearnedGuess(seed=seed)
    net.set_normalization(feat)
    return net


@pytest.mark.parametrize("batch", [256, 2048])
def test_gradients_match_oracle(fvs, torch_cuda, batch):
    torch = torch_cuda
    arr, dev, feat, lab, st = _problem_set(fvs, torch, batch, 12)
    net = _net_with_normalization(fvs, feat)
    p = net.master().astype(np.float64)
    g, loss = net.gradients(feat, lab, batch)
    F, L = feat.cpu().numpy(), lab.cpu().numpy().astype(np.float64)
    rloss, rg = mlp.loss_and_grad(p, F, L, bf16_operands=True)
    assert abs(loss - rloss) <= 1e-4 * rloss
    for lo, hi, name in [(mlp.OFF_W1, mlp.OFF_B1, "W1"), (mlp.OFF_B1, mlp.OFF_W2, "b1"),
                         (mlp.OFF_W2, mlp.OFF_B2, "W2"), (mlp.OFF_B2, mlp.OFF_W3, "b2"),
                         (mlp.OFF_W3, mlp.OFF_B3, "w3"), (mlp.OFF_B3, mlp.N_PARAMS, "b3")]:
        d = np.linalg.norm(g[lo:hi] - rg[lo:hi]) / np.linalg.norm(rg[lo:hi])
        assert d < 5e-3, (name, d)
    # and against the unrounded float64 network, within bfloat16's error
    _, rg64 = mlp.loss_and_grad(p, F, L)
    d = np.linalg.norm(g - rg64) / np.linalg.norm(rg64)
    assert d < 3e-2, d


def test_forward_matches_oracle(fvs, torch_cuda):
    torch = torch_cuda
    n = 3000  # not a multiple of the 128-row tile
    arr, dev, feat, lab, st = _problem_set(fvs, torch, n, 13)
    net = _net_with_normalization(fvs, feat)
    y = torch.empty(n, dtype=torch.float32, device="cuda")
    net.predict(feat, y)
    torch.cuda.synchronize()
    ref = mlp.forward(net.master().astype(np.float64), feat.cpu().numpy(), bf16_operands=True)
    err = np.abs(y.cpu().numpy() - ref)
    assert err.max() < 2e-3 * max(1.0, np.abs(ref).max()), err.max()


def test_adam_first_step_matches_oracle(fvs, torch_cuda):
    torch = torch_cuda
    arr, dev, feat, lab, st = _problem_set(fvs, torch, 1, 14)
    # every row the same problem: any sampled batch has that row's gradient
    feat_rep = feat.repeat(4096, 1).contiguous()
    lab_rep = lab.repeat(4096).contiguous()
    net = fvs.LearnedGuess(seed=5)
    p0 = net.master().astype(np.float64)
    g, _ = net.gradients(feat_rep, lab_rep, 256)
    net.train(feat_rep, lab_rep, steps=1, batch=256, lr=1e-3, seed=3)
    p1 = net.master().astype(np.float64)
    ref, _, _ = mlp.adam_step(p0, g.astype(np.float64), np.zeros(mlp.N_PARAMS),
                              np.zeros(mlp.N_PARAMS), 1, 1e-3)
    big = np.abs(g) > 1e-5  # tiny gradients: eps and rounding decide the step
    np.testing.assert_allclose(p1[big], ref[big], rtol=0, atol=2e-6)
    assert np.all(p1[:mlp.OFF_W1] == p0[:mlp.OFF_W1])


def test_training_cuts_newton_iterations(fvs, torch_cuda):
    torch = torch_cuda
    arr, dev, feat, lab, st = _problem_set(fvs, torch, 1 << 18, 21)
    ok = st == 1
    feat, lab = feat[ok].contiguous(), lab[ok].contiguous()
    net = _net_with_normalization(fvs, feat)
    first = net.train(feat, lab, steps=50, batch=8192, lr=1e-3, seed=1)
    net.train(feat, lab, steps=1500, batch=8192, lr=1e-3, seed=2)
    last = net.train(feat, lab, steps=50, batch=8192, lr=1e-3, seed=3)
    assert last < 0.1 * first, (first, last)
    # held-out problems, tolerance 1e-12
    n = 100000
    test = [torch.from_numpy(a).cuda() for a in workloads.riemann_samples(n, seed=99)]
    stats = {}
    for guess in ("mean", "pvrs_tr", "mlp"):
        m = fvs.make_method("godunov", guess=guess, tolerance=1e-12, max_iterations=200,
                            mlp_params=net.params_device_ptr() if guess == "mlp" else None)
        ps = torch.empty(n, dtype=torch.float64, device="cuda")
        it = torch.empty(n, dtype=torch.int32, device="cuda")
        s = torch.empty_like(it)
        fvs.exact_riemann_star(m, *test, ps, None, it, s)
        torch.cuda.synchronize()
        stats[guess] = (float(it.double().mean()), float((s == 2).double().mean()),
                        float((s == 0).double().mean()), ps.cpu().numpy(), s.cpu().numpy())
    mean_it, pvrs_it, mlp_it = stats["mean"][0], stats["pvrs_tr"][0], stats["mlp"][0]
    summary = {k: v[:3] for k, v in stats.items()}
    print("newton iterations / fallback rate / failures:", summary)
    assert mlp_it < 0.75 * mean_it, summary
    # the gain over PVRS/TR, the start value the solver would use without
    # the network: fewer Newton steps per problem at this tolerance
    assert mlp_it < 0.95 * pvrs_it, summary
    assert stats["mlp"][2] <= stats["mean"][2]
    conv = (stats["mlp"][4] != 0) & (stats["mean"][4] != 0)
    # same root from either start value; near-vacuum p* (down to 1e-28 here)
    # is only determined to the solver's tolerance relative to max(pL, pR)
    pref = np.maximum(test[2].cpu().numpy(), test[5].cpu().numpy())[conv]
    diff = np.abs(stats["mlp"][3][conv] - stats["mean"][3][conv])
    assert np.all(diff <= 1e-10 * np.abs(stats["mean"][3][conv]) + 1e-12 * pref)
