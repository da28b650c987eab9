"""Turn scheduler: the learned MLP's inference and training kernels against a
PyTorch fp32 reference, and bit-exact results under every schedule (the
schedule only changes the order of reduction)."""
from __future__ import annotations

import hashlib
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def torch_mlp(w: np.ndarray):
    """Parameter tensors of the packed layout W1 b1 W2 b2 W3 b3."""
    t = torch.tensor(w, dtype=torch.float32)
    shapes = [(64, 16), (64,), (64, 64), (64,), (3, 64), (3,)]
    out, k = [], 0
    for s in shapes:
        n = int(np.prod(s))
        out.append(t[k:k + n].reshape(s).clone().requires_grad_(True))
        k += n
    return out


def torch_forward(params, x):
    w1, b1, w2, b2, w3, b3 = params
    h1 = torch.relu(x @ w1.T + b1)
    h2 = torch.relu(h1 @ w2.T + b2)
    return torch.sigmoid(h2 @ w3.T + b3)


def random_problem(n: int, seed: int):
    rng = np.random.default_rng(seed)
    train = importlib.import_module("lambdavm-rust_gb300.train_policy")
    w = train.init_weights(seed)
    w[-3:] = rng.normal(0, 0.5, 3).astype(np.float32)  # non-zero output biases
    x = rng.uniform(-0.2, 1.0, (n, 16)).astype(np.float32)
    t = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    sw = rng.uniform(0.1, 2.0, n).astype(np.float32)
    return w, x, t, sw


def test_policy_forward_matches_torch(hvm):
    w, x, _, _ = random_problem(1000, 3)
    y = hvm.policy_forward(w, x)
    ref = torch_forward(torch_mlp(w), torch.tensor(x)).detach().numpy()
    # fp32 with a fast exponential in the sigmoid: 1e-5 absolute on outputs in (0, 1).
    np.testing.assert_allclose(y, ref, atol=1e-5, rtol=0)


@pytest.mark.parametrize("n", [1, 63, 64, 1000, 20000])
def test_policy_grad_matches_torch(hvm, n):
    w, x, t, sw = random_problem(n, 5 + n)
    loss, g = hvm.policy_grad(w, x, t, sw)
    params = torch_mlp(w)
    xt, tt, st = torch.tensor(x), torch.tensor(t), torch.tensor(sw)
    y = torch_forward(params, xt)
    ref_loss = (st[:, None] * (y - tt) ** 2).sum() / st.sum()
    ref_loss.backward()
    ref_g = torch.cat([p.grad.reshape(-1) for p in params]).numpy()
    # fp32 sums in a different order: relative 1e-4 on the loss, and
    # 1e-5 * max|grad| + 1e-3 relative per component.
    assert abs(loss - ref_loss.item()) <= 1e-4 * abs(ref_loss.item()) + 1e-7
    scale = np.abs(ref_g).max()
    np.testing.assert_allclose(g, ref_g, atol=1e-5 * scale, rtol=1e-3)


def test_policy_train_fits(hvm):
    # A target the MLP can represent: its own outputs under other weights.
    w_true, x, _, sw = random_problem(4096, 11)
    t = hvm.policy_forward(w_true, x)
    train = importlib.import_module("lambdavm-rust_gb300.train_policy")
    w0 = train.init_weights(12)
    loss0, _ = hvm.policy_grad(w0, x, t, sw)
    w, loss = hvm.policy_train(w0, x, t, sw, epochs=1500, lr=3e-3)
    loss_after, _ = hvm.policy_grad(w, x, t, sw)
    assert np.all(np.isfinite(w))
    assert loss_after < 0.05 * loss0, (loss0, loss, loss_after)


def test_policy_train_matches_torch_adam(hvm):
    # Five full-batch Adam steps against torch.optim.Adam (same betas, eps).
    w, x, t, sw = random_problem(500, 21)
    got, _ = hvm.policy_train(w, x, t, sw, epochs=5, lr=1e-2)
    params = torch_mlp(w)
    opt = torch.optim.Adam(params, lr=1e-2, betas=(0.9, 0.999), eps=1e-8)
    xt, tt, st = torch.tensor(x), torch.tensor(t), torch.tensor(sw)
    for _ in range(5):
        opt.zero_grad()
        y = torch_forward(params, xt)
        ((st[:, None] * (y - tt) ** 2).sum() / st.sum()).backward()
        opt.step()
    ref = torch.cat([p.detach().reshape(-1) for p in params]).numpy()
    # Adam's first steps move each weight by about lr * sign(g): compare to a
    # small fraction of the step.
    np.testing.assert_allclose(got, ref, atol=2e-4, rtol=0)


def _canon_sha(hvm, text: str) -> str:
    return hashlib.sha256(hvm.canonical(text).encode()).hexdigest()


SCHEDULES = [
    (0.0, -1, -1, 0.0, 0.0, 0.0),       # shortest turns, stop early, minimal static share
    (1.0, 1.0, -1, 1.0, 1.0, 1.0),      # longest turns, never stop early, full share
    (0.4, 0.5, 0.5, 0.6, 0.3, 0.7),
    (-1, -1, -1, -1, -1, -1),           # every entry keeps the fixed choice
]


@pytest.mark.parametrize("case", ["tree_sum_d12", "bitonic_sort_2p8", "skewed_fold_2p10", "countdown_100000"])
def test_schedules_are_bit_exact(hvm, workloads, config_goldens, case):
    code = {
        "tree_sum_d12": lambda: workloads.tree_sum(12),
        "bitonic_sort_2p8": lambda: workloads.bitonic_sort(8),
        "skewed_fold_2p10": lambda: workloads.skewed_fold(10),
        "countdown_100000": lambda: workloads.countdown(100000),
    }[case]()
    gold = config_goldens[case]
    rng = np.random.default_rng(7)
    train = importlib.import_module("lambdavm-rust_gb300.train_policy")
    rand_w = train.init_weights(9)
    rand_w[-3:] = rng.normal(0, 2.0, 3).astype(np.float32)
    with hvm.Runtime(device=0, trace_cap=4096) as rt:
        rt.load(code)
        for const in SCHEDULES:
            rt.set_policy(hvm.POLICY_CONSTANT, constants=const)
            st = rt.run()
            assert st.itrs == gold["itrs"], const
            assert _canon_sha(hvm, rt.result()) == gold["canonical_sha256"], const
        rt.set_policy(hvm.POLICY_LEARNED, weights=rand_w)
        st = rt.run()
        assert st.itrs == gold["itrs"]
        assert _canon_sha(hvm, rt.result()) == gold["canonical_sha256"]
        tr = rt.trace()
        assert tr and all(0.0 <= o <= 1.0 for r in tr for o in r["outputs"])
        assert all(np.isfinite(r["features"]).all() for r in tr)
        # A per-turn script (the local search's probe): random decisions at
        # every turn, then one decision at a single turn.
        script = rng.uniform(0.0, 1.0, 3 * 64).astype(np.float32)
        for s in (script, [-1.0] * 6 + [1.0, 0.0, -1.0]):
            rt.set_policy(hvm.POLICY_SCRIPT, weights=s)
            st = rt.run()
            assert st.itrs == gold["itrs"]
            assert _canon_sha(hvm, rt.result()) == gold["canonical_sha256"]
        # The decision a script gives at turn 0 is the one the trace records.
        rt.set_policy(hvm.POLICY_SCRIPT, weights=[0.3, 0.0, -1.0])  # 512 rounds (under the 1024 cap)
        rt.run()
        assert rt.trace()[0]["outputs"][:2] == pytest.approx([0.3, 0.0], abs=1e-6)


def test_committed_policy_on_skewed_fold(hvm, workloads, config_goldens):
    train = importlib.import_module("lambdavm-rust_gb300.train_policy")
    w = train.load_weights()
    gold = config_goldens["skewed_fold_2p18"]
    with hvm.Runtime(device=0) as rt:
        rt.load(workloads.skewed_fold(18))
        rt.set_policy(hvm.POLICY_LEARNED, weights=w)
        st = rt.run()
        assert st.itrs == gold["itrs"]
        assert _canon_sha(hvm, rt.result()) == gold["canonical_sha256"]


def test_policy_errors(hvm):
    with hvm.Runtime(device=0) as rt:
        with pytest.raises(hvm.HvmError):
            rt.set_policy(hvm.POLICY_LEARNED, weights=[0.0] * 10)
        with pytest.raises(hvm.HvmError):
            rt.set_policy(7)
        with pytest.raises(hvm.HvmError):
            rt.set_policy(hvm.POLICY_SCRIPT, weights=[0.5] * 4)  # not 3 per turn
        bad = np.zeros(hvm.POLICY_PARAMS, dtype=np.float32)
        bad[5] = np.nan
        with pytest.raises(hvm.HvmError):
            rt.set_policy(hvm.POLICY_LEARNED, weights=bad)
