"""Adjoint of the non-cyclic solve (pbt_adjoint_noncyclic) and its
torch.autograd binding.  lambda is checked against the oracle applied to the
block-transposed system (At_q = C_{q-1}^T, Bt_q = B_q^T, Ct_q = A_{q+1}^T),
the gradient blocks against -lambda x^T, and the whole binding against
central finite differences (h = 1e-6) of L = sum(w * x)."""
import numpy as np
import pytest
import torch

import pascal_btdma_gb300 as pbt
from pascal_btdma_gb300 import synth
from pascal_btdma_gb300.synth import Workload
from conftest import per_system_relerr
from gpu_util import oracle_solve, to_dev

pytestmark = pytest.mark.gpu
TOL = 1e-12


def transposed(w):
    """The block-transposed workload M^T (reference layout)."""
    m, nsys, N = w.m, w.nsys, w.nrow
    A4 = w.A.reshape(m, m, N, nsys)  # [j, i, row, sys]
    B4 = w.B.reshape(m, m, N, nsys)
    C4 = w.C.reshape(m, m, N, nsys)
    At = np.zeros_like(A4)
    Ct = np.zeros_like(C4)
    At[:, :, 1:] = C4.transpose(1, 0, 2, 3)[:, :, :-1]
    Ct[:, :, :-1] = A4.transpose(1, 0, 2, 3)[:, :, 1:]
    Bt = np.ascontiguousarray(B4.transpose(1, 0, 2, 3))
    return Workload(m, nsys, N, At.reshape(-1).copy(), Bt.reshape(-1).copy(), Ct.reshape(-1).copy(), w.D.copy())


def run_adjoint(w, nseg, prec, g):
    a, b, c, d = to_dev(w.arrays, "cuda:0")
    x = d.clone()
    lam = torch.from_numpy(g).to("cuda:0")
    da, db, dc = torch.empty_like(a), torch.empty_like(b), torch.empty_like(c)
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(w.m, w.nsys, w.nrow, nseg, precision=prec)
        pbt.solve_noncyclic(plan, a, b, c, x, w.m, w.nsys, w.nrow)
        pbt.adjoint_noncyclic(plan, a, b, c, x, lam, da, db, dc)
        assert plan.status() == 0
    assert torch.equal(a.cpu(), torch.from_numpy(w.A))
    return x.cpu().numpy(), lam.cpu().numpy(), da.cpu().numpy(), db.cpu().numpy(), dc.cpu().numpy()


@pytest.mark.parametrize("m,nsys,nrow,nseg", [(1, 37, 10, 1), (2, 65, 9, 3), (3, 33, 40, 1), (4, 96, 64, 8),
                                              (5, 70, 24, 1), (5, 64, 256, 16), (6, 40, 2, 1), (7, 64, 12, 1),
                                              (7, 33, 2, 1), (8, 9, 16, 2), (8, 64, 16, 1), (9, 35, 9, 1),
                                              (10, 5, 12, 1), (10, 64, 3, 1)])
@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_adjoint_matches_transposed_oracle(cuda, m, nsys, nrow, nseg, prec):
    w = synth.dominant(m, nsys, nrow, seed=300 + m, delta=1.5)
    g = np.random.default_rng(m).uniform(-1, 1, nsys * nrow * m)
    x, lam, da, db, dc = run_adjoint(w, nseg, prec, g)
    wt = transposed(w)
    wt.D[:] = g
    ref = oracle_solve(wt, nseg)
    assert per_system_relerr(m, nsys, nrow, lam, ref.D) <= TOL
    # gradient blocks: dB_q = -lambda_q x_q^T, dC_q = -lambda_q x_{q+1}^T, dA_q = -lambda_q x_{q-1}^T
    L = lam.reshape(m, nrow, nsys)
    X = x.reshape(m, nrow, nsys)
    eB = -np.einsum("irs,jrs->jirs", L, X)
    eC = np.zeros_like(eB)
    eC[:, :, :-1] = -np.einsum("irs,jrs->jirs", L[:, :-1], X[:, 1:])
    eA = np.zeros_like(eB)
    eA[:, :, 1:] = -np.einsum("irs,jrs->jirs", L[:, 1:], X[:, :-1])
    scale = np.abs(eB).max()
    for got, exp in ((db, eB), (dc, eC), (da, eA)):
        assert np.abs(got.reshape(m, m, nrow, nsys) - exp).max() <= 1e-13 * scale


@pytest.mark.parametrize("m,nseg,prec", [(4, 1, "fp64"), (4, 8, "fp64"), (4, 1, "ff"), (4, 8, "ff"),
                                         (7, 1, "fp64"), (8, 1, "ff"), (9, 2, "fp64"), (10, 1, "fp64"),
                                         (10, 1, "ff")])
def test_autograd_finite_differences(cuda, m, nseg, prec):
    """L = sum(w * x), x = M^{-1} d; autograd gradients vs central differences
    on 64 random entries of each of A, B, C, d (h = 1e-6, FP64 solves)."""
    nsys, nrow = 64, 64
    wl = synth.dominant(m, nsys, nrow, seed=77, delta=1.5)
    dev = torch.device(cuda)
    A, B, C, d = (torch.from_numpy(t).to(dev).requires_grad_(True) for t in wl.arrays)
    wts = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, nsys * nrow * m)).to(dev)
    plan = pbt.BtdmaGpuPlan().create(m, nsys, nrow, nseg, precision=prec)
    x = pbt.BlockTridiagonalSolve.apply(A, B, C, d, plan)
    loss = (wts * x).sum()
    loss.backward()
    plan64 = pbt.BtdmaGpuPlan().create(m, nsys, nrow, nseg, precision="fp64")

    def L(arrs):
        xx = arrs[3].clone()
        pbt.solve_noncyclic(plan64, arrs[0], arrs[1], arrs[2], xx, m, nsys, nrow)
        return float((wts * xx).sum())

    base = [t.detach().clone() for t in (A, B, C, d)]
    rng = np.random.default_rng(2)
    h = 1e-6
    for which, grad in enumerate((A.grad, B.grad, C.grad, d.grad)):
        n = base[which].numel()
        idx = rng.choice(n, size=64, replace=False)
        if which in (0, 2):  # A_0 and C_{N-1} never enter: keep them in the sample, their gradient is 0
            pass
        fd = np.empty(64)
        for k, e in enumerate(idx):
            plus = [t.clone() for t in base]
            minus = [t.clone() for t in base]
            plus[which].view(-1)[e] += h
            minus[which].view(-1)[e] -= h
            fd[k] = (L(plus) - L(minus)) / (2 * h)
        an = grad.view(-1)[torch.from_numpy(idx).to(dev)].cpu().numpy()
        err = np.abs(fd - an).max()
        assert err <= 1e-6 * max(1.0, np.abs(an).max()), (which, err)
    plan.destroy()
    plan64.destroy()


def test_adjoint_rejects_inplace_and_bad_sizes(cuda):
    w = synth.dominant(3, 32, 12, seed=1, delta=2.0)
    a, b, c, d = to_dev(w.arrays, cuda)
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(3, 32, 12, 1, inplace=True)
        with pytest.raises(NotImplementedError, match="INPLACE"):
            pbt.adjoint_noncyclic(plan, a, b, c, d, d.clone())
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(3, 32, 12, 1)
        with pytest.raises(ValueError, match="do not match"):
            pbt.adjoint_noncyclic(plan, a, b, c, d, d.clone(), m=3, nsys=32, nrow=13)


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_adjoint_full_size_finite_differences(cuda, prec):
    """The adjoint workload at its full size: m = 4, nsys = 16384, N = 512,
    P = 8, delta = 1.5, L = sum(w . x) with w iid U[-1, 1).  dL/dA, dL/dB,
    dL/dC, dL/dd from the adjoint kernel against central differences
    (h = 1e-6, FP64 solves) on 64 random entries of each; entries are
    perturbed in place and restored.  The system index is fastest in the
    layout, so entry e belongs to system e % nsys."""
    m, nsys, nrow, nseg = 4, 16384, 512, 8
    wl = synth.dominant(m, nsys, nrow, seed=5, delta=1.5)
    dev = torch.device(cuda)
    A, B, C, d = (torch.from_numpy(t).to(dev) for t in wl.arrays)
    wts = torch.from_numpy(np.random.default_rng(3).uniform(-1, 1, nsys * nrow * m)).to(dev)
    with pbt.BtdmaGpuPlan() as plan, pbt.BtdmaGpuPlan() as plan64:
        plan.create(m, nsys, nrow, nseg, precision=prec)
        plan64.create(m, nsys, nrow, nseg, precision="fp64")
        x = d.clone()
        pbt.solve_noncyclic(plan, A, B, C, x, m, nsys, nrow)
        lam = wts.clone()
        dA, dB, dC = torch.empty_like(A), torch.empty_like(B), torch.empty_like(C)
        pbt.adjoint_noncyclic(plan, A, B, C, x, lam, dA, dB, dC)
        assert plan.status() == 0
        xx = torch.empty_like(d)
        w2 = wts.view(-1, nsys)

        def L(sys):
            # An entry of system `sys` moves only that system's x, so L's
            # change is that system's share of the sum: summing only it
            # keeps the rounding of the other 16383 systems out of the
            # difference quotient.
            xx.copy_(d)
            pbt.solve_noncyclic(plan64, A, B, C, xx, m, nsys, nrow)
            return float(torch.dot(w2[:, sys], xx.view(-1, nsys)[:, sys]))

        rng = np.random.default_rng(4)
        h = 1e-6
        for arr, grad in ((A, dA), (B, dB), (C, dC), (d, lam)):
            flat = arr.view(-1)
            idx = rng.choice(flat.numel(), size=64, replace=False)
            fd = np.empty(64)
            for k, e in enumerate(idx.tolist()):
                v = float(flat[e])
                flat[e] = v + h
                lp = L(e % nsys)
                flat[e] = v - h
                lm = L(e % nsys)
                flat[e] = v
                fd[k] = (lp - lm) / (2 * h)
            an = grad.view(-1)[torch.from_numpy(idx).to(dev)].cpu().numpy()
            err = np.abs(fd - an).max()
            assert err <= 1e-6 * max(1.0, np.abs(an).max()), err
