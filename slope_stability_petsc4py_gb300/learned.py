"""Learned branch proposal for the 3D return mapping (trained and run on the GPU).

The reference decides every point's return branch inside one divergent kernel
(``src/slope_stability/cython/constitutive_3D_kernel.h:116-350``).  Here a 6 -> 32 -> 32 -> 5
ReLU network proposes the branch from cheap FP32 invariants of the trial strain for the points
that the binned return mapping's FP32 elastic screen cannot settle (near or past the yield
surface); those points are binned by the proposal and the exact FP64 decision pass runs bin by
bin, so each warp mostly follows one branch's checks.  The exact kernels still decide and compute
every result: a wrong proposal costs time, never accuracy.

Training data are (features, branch) pairs of the screen-listed points, emitted by the exact
return mapping on a sequence of continuation states (``collect_training_data``).  Training runs on the GPU through the library's
own kernels: ``ssp_mlp_loss_grad`` (forward and backward of a batch), ``ssp_mlp_adam``.
"""

from __future__ import annotations

import numpy as np

from . import _lib
from .distributed_tangent import overlap_strain_device

N_PARAMS = 1445
SHAPES = (("W1", (32, 6)), ("b1", (32,)), ("W2", (32, 32)), ("b2", (32,)), ("W3", (5, 32)), ("b3", (5,)))
BRANCHES = ("elastic", "smooth", "left_edge", "right_edge", "apex")


def init_params(seed: int = 0) -> np.ndarray:
    """He-uniform weights, zero biases, as one FP32 vector in the kernels' layout."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in SHAPES:
        if name.startswith("W"):
            bound = np.sqrt(6.0 / shape[1])
            parts.append(rng.uniform(-bound, bound, size=shape).ravel())
        else:
            parts.append(np.zeros(shape))
    return np.concatenate(parts).astype(np.float32)


def features(E, c_bar, sin_phi, shear, lame):
    """FP32 features [n, 6] of AoS trial strains E [n, 6] (all CUDA tensors)."""
    t = _lib.require_cuda()
    n = int(E.shape[0])
    X = t.empty((n, 6), dtype=t.float32, device="cuda")
    _lib.call("ssp_branch_features", _lib.ptr(E), _lib.ptr(c_bar), _lib.ptr(sin_phi), _lib.ptr(shear), _lib.ptr(lame), n,
              _lib.ptr(X), _lib.stream_handle())
    return X


def exact_branches(E, c_bar, sin_phi, shear, lame):
    """Branch codes the exact return mapping takes, int8 [n]."""
    t = _lib.require_cuda()
    n = int(E.shape[0])
    S = t.empty((n, 6), dtype=t.float64, device="cuda")
    br = t.empty(n, dtype=t.int8, device="cuda")
    _lib.call("ssp_constitutive_3d_branch", _lib.ptr(E), _lib.ptr(c_bar), _lib.ptr(sin_phi), _lib.ptr(shear),
              _lib.ptr(lame), n, _lib.ptr(S), _lib.ptr(br), _lib.stream_handle())
    return br


def screen_listed(E, c_bar, sin_phi, shear, lame):
    """(indices of the points the binned return mapping's FP32 elastic screen cannot settle, branch
    codes of all points), from one ssp_constitutive_3d_sds_binned call."""
    t = _lib.require_cuda()
    n = int(E.shape[0])
    S = t.empty((n, 6), dtype=t.float64, device="cuda")
    DS = t.empty((n, 36), dtype=t.float64, device="cuda")
    br = t.empty(n, dtype=t.int8, device="cuda")
    scratch = t.empty(3 * n + 4, dtype=t.int32, device="cuda")
    _lib.call("ssp_constitutive_3d_sds_binned", _lib.ptr(E), _lib.ptr(c_bar), _lib.ptr(sin_phi), _lib.ptr(shear),
              _lib.ptr(lame), n, _lib.ptr(S), _lib.ptr(DS), _lib.ptr(br), _lib.ptr(scratch), _lib.stream_handle())
    return scratch[4: 4 + int(scratch[0])].long(), br


def collect_training_data(op, states, listed_only: bool = True, max_per_state: int | None = None, seed: int = 0):
    """(features, labels) from the exact return mapping over continuation states [(lam, U), ...].
    With listed_only, only the points the elastic screen lists: the ones the learned return
    mapping asks the network about.  max_per_state: a seeded uniform sample of at most that many
    of a state's points (large meshes list millions per state)."""
    t = _lib.require_cuda()
    pat = op.owned_tangent_pattern
    Xs, ys = [], []
    gen = t.Generator(device="cuda")
    gen.manual_seed(seed)
    for lam, U in states:
        op.reduction(lam)
        E = overlap_strain_device(pat, U)
        d = op._dev
        args = (E, op._owned_overlap_c_bar, op._owned_overlap_sin_phi, d["shear"], d["lame"])
        X = features(*args)
        if listed_only:
            pick, br = screen_listed(*args)
        else:
            pick, br = t.arange(X.shape[0], device="cuda"), exact_branches(*args)
        if max_per_state is not None and pick.numel() > max_per_state:
            pick = pick.index_select(0, t.randperm(pick.numel(), device="cuda", generator=gen)[:max_per_state])
        Xs.append(X.index_select(0, pick))
        ys.append(br.index_select(0, pick))
    return t.cat(Xs), t.cat(ys)


class BranchProposal:
    """The proposal network: FP32 parameters on the device, GPU training and prediction."""

    def __init__(self, params=None, seed: int = 0):
        t = _lib.require_cuda()
        p = init_params(seed) if params is None else np.asarray(params, dtype=np.float32)
        if p.size != N_PARAMS:
            raise ValueError(f"expected {N_PARAMS} parameters")
        self.params = t.as_tensor(p, device="cuda").contiguous()
        self.history = []

    def loss_grad(self, X, y):
        """(summed loss, summed gradient, argmax hits) of a batch, from ssp_mlp_loss_grad."""
        t = _lib.require_cuda()
        grad = t.empty(N_PARAMS, dtype=t.float32, device="cuda")
        loss = t.empty(1, dtype=t.float32, device="cuda")
        hits = t.empty(1, dtype=t.int32, device="cuda")
        _lib.call("ssp_mlp_loss_grad", _lib.ptr(self.params), _lib.ptr(X), _lib.ptr(y), int(X.shape[0]), _lib.ptr(grad),
                  _lib.ptr(loss), _lib.ptr(hits), _lib.stream_handle())
        return loss, grad, hits

    def train(self, X, y, *, epochs: int = 4, batch: int = 65536, lr: float = 3e-3, seed: int = 0):
        """Adam on shuffled mini-batches; returns the per-epoch (mean loss, accuracy) history."""
        t = _lib.require_cuda()
        n = int(X.shape[0])
        m = t.zeros(N_PARAMS, dtype=t.float32, device="cuda")
        v = t.zeros(N_PARAMS, dtype=t.float32, device="cuda")
        gen = t.Generator(device="cuda")
        gen.manual_seed(seed)
        step = 0
        for ep in range(epochs):
            perm = t.randperm(n, device="cuda", generator=gen)
            tot_loss = t.zeros(1, dtype=t.float64, device="cuda")
            tot_hits = t.zeros(1, dtype=t.int64, device="cuda")
            for s in range(0, n, batch):
                idx = perm[s:s + batch]
                Xb, yb = X.index_select(0, idx).contiguous(), y.index_select(0, idx).contiguous()
                loss, grad, hits = self.loss_grad(Xb, yb)
                step += 1
                _lib.call("ssp_mlp_adam", _lib.ptr(self.params), _lib.ptr(grad), _lib.ptr(m), _lib.ptr(v), step, lr, 0.9,
                          0.999, 1e-8, 1.0 / int(idx.numel()), _lib.stream_handle())
                tot_loss += loss.double()
                tot_hits += hits.long()
            self.history.append((float(tot_loss.item()) / n, float(tot_hits.item()) / n))
        return self.history

    def predict(self, X, *, bf16: bool = True, tensor_cores: bool = True):
        """Argmax branch of every feature row: BF16 on the tensor cores (the binning's inference),
        BF16 or FP32 on the CUDA cores."""
        t = _lib.require_cuda()
        pred = t.empty(int(X.shape[0]), dtype=t.int8, device="cuda")
        mode = (2 if tensor_cores else 1) if bf16 else 0
        _lib.call("ssp_mlp_predict", _lib.ptr(self.params), _lib.ptr(X), int(X.shape[0]), mode, _lib.ptr(pred),
                  _lib.stream_handle())
        return pred

    def accuracy(self, X, y, *, bf16: bool = True) -> float:
        return float((self.predict(X, bf16=bf16) == y).float().mean().item())

    def state(self) -> np.ndarray:
        return self.params.cpu().numpy().copy()


def proposal_bins(scratch, n: int):
    """The learned return mapping's point lists, read from its scratch after a call on n points:
    the points the elastic screen listed (in point order) and the five bins of proposed branches
    over them (layout of ``ssp_constitutive_3d_sds_learned``)."""
    listed = scratch[4: 4 + int(scratch[0])].long()
    cnt = scratch[4 + 3 * n: 9 + 3 * n].cpu().numpy()
    base = 12 + 3 * n
    bins = [scratch[base + k * n: base + k * n + int(cnt[k])].long() for k in range(5)]
    return listed, bins


def warp_branch_mix(branches, order=None) -> float:
    """Mean number of distinct branches per 32-point warp when points run in ``order``: the
    divergence the return-mapping warps see (1.0 = no divergence)."""
    t = _lib.torch()
    b = branches if order is None else branches.index_select(0, order)
    n = (b.numel() // 32) * 32
    w = b[:n].view(-1, 32).long()
    present = t.zeros((w.shape[0], 5), dtype=t.bool, device=w.device)
    present.scatter_(1, w, True)
    return float(present.sum(dim=1).float().mean().item())
