"""QoI-bounded retrieval of several fields (velocity components, density).

Two drivers retrieve the fields until a pointwise bound on a derived quantity
of interest holds: max_i |Q(V~(i)) - Q(V(i))| <= tau.

* ``halving_retrieve`` -- the reference's uniform-tightening loop
  (app/GE/sequential/halving_Vtot.cpp:31-84 and :153-189): every field is
  retrieved to its own L-inf bound eb_f (SignExclude greedy interpreter,
  MaxErrorEstimatorHB); the pointwise QoI bound is evaluated with the
  reference's error propagation rules (include/qoi_utils.hpp:18-48, :95-98;
  for |V| by the device kernel behind ``prodm_qoi_ge_bounds``, bit for bit
  the reference's V_TOT estimate); while its maximum exceeds tau, all eb_f shrink by 1.5 until the bound at
  the worst point holds, and the fields are retrieved again (at most 5 times).

* ``guided_retrieve`` -- per-(field, level) bitplane budgets from the QoI's
  sensitivity. For the hierarchical basis the recomposition R has
  non-negative weights, so the error of field f at point i obeys
  |dV_f(i)| <= sum_l r_l(i) e_fl, with e_fl the L-inf error bound of level l
  and r_l(i) = sum over level-l coefficients j of R(i, j) the level's
  influence at i (r_l = R applied to the level-l indicator). The pointwise
  QoI bound uses these per-point field bounds in the same propagation rules.
  At the worst point i*, the gradient of Q(i*) with respect to the level
  coefficients -- the adjoint recomposition applied to dQ/dV(i*) at i* --
  has per-level L1 norms |dQ/dV_f(i*)| r_l(i*); they weigh each candidate
  bitplane's error reduction against its bytes in one greedy over all
  (field, level) pairs, until the planned bound holds; the fields are then
  retrieved and the bound is re-evaluated on the new reconstruction.

Both drivers report the retrieved bytes, the rigorous bound and the achieved
error (when the original fields are given). All field arithmetic runs on the
device; the planning loop is host logic over at most fields x levels x
bitplanes entries.
"""
import heapq
import math

import numpy as np
import torch

from . import api


# ---------------------------------------------------------------------------
# error propagation (include/qoi_utils.hpp:18-48, :95-98), elementwise
# ---------------------------------------------------------------------------
def bound_x_square(x, eb):
    return 2.0 * x.abs() * eb + eb * eb


def bound_sqrt(x, eb):
    # x == 0 -> sqrt(eb); x > eb -> eb / (sqrt(x - eb) + sqrt(x)); else eb / sqrt(x)
    safe = torch.where(x > 0, x, torch.ones_like(x))
    big = eb / (torch.sqrt(torch.clamp(x - eb, min=0.0)) + torch.sqrt(safe))
    small = eb / torch.sqrt(safe)
    out = torch.where(x > eb, big, small)
    return torch.where(x == 0, torch.sqrt(eb), out)


def bound_multiplication(x, y, eb_x, eb_y):
    return x.abs() * eb_y + y.abs() * eb_x + eb_x * eb_y


def qoi_value(kind, V, rho=None):
    vv = V[0] * V[0] + V[1] * V[1] + V[2] * V[2]
    if kind == "vmag":
        return torch.sqrt(vv)
    return 0.5 * rho * vv


def qoi_bound(kind, V, ebV, rho=None, eb_rho=None):
    """Pointwise bound on |Q(true) - Q(V)| given |V_f(true) - V_f| <= ebV[f]
    (scalars or per-point tensors), all in float64."""
    e2 = bound_x_square(V[0], ebV[0]) + bound_x_square(V[1], ebV[1]) + bound_x_square(V[2], ebV[2])
    vv = V[0] * V[0] + V[1] * V[1] + V[2] * V[2]
    if kind == "vmag":
        return bound_sqrt(vv, e2)
    return 0.5 * bound_multiplication(rho, vv, eb_rho, e2)


def value_range(x):
    return float(x.max() - x.min())


# ---------------------------------------------------------------------------
# fields
# ---------------------------------------------------------------------------
class _Field:
    def __init__(self, data, L, B, encoder):
        self.shape = tuple(data.shape)
        self.mdr = api.MDRField(self.shape, data.dtype, L, B, encoder, "hierarchical", "max")
        self.mdr.refactor(data.contiguous())
        self.sizes, self.bounds, _ = self.mdr.level_info()
        self.L, self.B = L, B
        # MaxErrorCollector tables: error bound of level l after b planes
        self.errs = np.stack([api.collect_max(float(b), B, data.dtype) for b in self.bounds])
        self.index = np.zeros(L + 1, np.int64)
        self.out = torch.empty(self.shape, dtype=data.dtype, device="cuda")

    def level_errors(self, index=None):
        idx = self.index if index is None else index
        return np.array([self.errs[l, idx[l]] for l in range(self.L + 1)])

    def bytes(self, index=None):
        idx = self.index if index is None else index
        return int(sum(int(self.sizes[l, :idx[l]].astype(np.int64).sum()) for l in range(self.L + 1)))

    def retrieve_planes(self, index):
        self.index = np.maximum(self.index, np.asarray(index, np.int64))
        self.mdr.retrieve_planes([int(v) for v in self.index], out=self.out)
        return self.out

    def retrieve_tolerance(self, eb):
        self.mdr.retrieve(eb, out=self.out, interpreter="sign_exclude", estimator="max_hb")
        self.index = self.mdr.index().astype(np.int64)
        return self.out


def _unpack(kind, fields):
    V = [f.out.double() for f in fields[:3]]
    rho = fields[3].out.double() if kind == "ke" else None
    return V, rho


def _achieved(kind, fields, originals):
    if originals is None:
        return None
    V, rho = _unpack(kind, fields)
    q = qoi_value(kind, V, rho)
    qo = qoi_value(kind, [o.double() for o in originals[:3]], originals[3].double() if kind == "ke" else None)
    return float((q - qo).abs().max())


# ---------------------------------------------------------------------------
# reference loop: uniform halving
# ---------------------------------------------------------------------------
def halving_retrieve(kind, data, tau, rel, L, B=32, encoder="grouped", max_iter=5):
    """data: [Vx, Vy, Vz] (+ [rho] for kind == "ke") device tensors. Returns a
    dict with bytes, bound, achieved error and iterations."""
    fields = [_Field(x, L, B, encoder) for x in data]
    ebs = [value_range(x) * rel for x in data]                     # halving_Vtot.cpp:99-103
    it, met, bound = 0, False, math.inf
    while not met and it < max_iter:
        it += 1
        for f, eb in zip(fields, ebs):
            f.retrieve_tolerance(eb)
        V, rho = _unpack(kind, fields)
        if kind == "vmag":
            # the reference's V_TOT estimate, evaluated by prodm_qoi_ge_bounds
            est, _, mx = api.qoi_ge_bounds([v.reshape(-1) for v in V], ebs[:3])
            bound = float(mx[0])
        else:
            est = qoi_bound(kind, V, ebs[:3], rho, ebs[3] if kind == "ke" else None)
            bound = float(est.max())
        if bound <= tau:
            met = True
            break
        # uniform decrease at the worst point (halving_Vtot.cpp:56-80)
        i = int(torch.argmax(est))
        Vi = [v.reshape(-1)[i:i + 1] for v in V]
        ri = rho.reshape(-1)[i:i + 1] if kind == "ke" else None
        e = bound
        while e > tau:
            ebs = [x / 1.5 for x in ebs]
            if kind == "vmag":
                e = float(api.qoi_ge_bounds(Vi, ebs[:3])[2][0])
            else:
                e = float(qoi_bound(kind, Vi, [torch.tensor(x, dtype=torch.float64, device="cuda") for x in ebs[:3]],
                                    ri, torch.tensor(ebs[3], dtype=torch.float64, device="cuda")))
    return {"bytes": sum(f.bytes() for f in fields), "bound": bound, "met": met, "iterations": it,
            "achieved": _achieved(kind, fields, data), "index": [f.index.tolist() for f in fields]}


# ---------------------------------------------------------------------------
# QoI-guided: per-(field, level) budgets
# ---------------------------------------------------------------------------
def level_influence(shape, L, dtype=torch.float32):
    """r_l = R 1_l for every level: stacked (L+1, N) device tensor."""
    el = api.level_dims(shape, L)[1].astype(np.int64)
    off = np.concatenate([[0], np.cumsum(el)])
    n = int(off[-1])
    rs = []
    for l in range(L + 1):
        ind = torch.zeros(n, dtype=dtype, device="cuda")
        ind[int(off[l]):int(off[l + 1])] = 1
        rs.append(api.recompose_packed(ind, shape, L).reshape(-1).double())
    return torch.stack(rs), off


def point_level_weights(shape, L, i, off, dtype=torch.float32):
    """per-level L1 norms of d V(i) / d(level coefficients): the adjoint
    recomposition of a unit gradient at point i"""
    g = torch.zeros(int(np.prod(shape)), dtype=dtype, device="cuda")
    g[i] = 1
    a = api.recompose_adjoint(g.reshape(shape), L).double().abs()
    return np.array([float(a[int(off[l]):int(off[l + 1])].sum()) for l in range(L + 1)])


def _pointwise_bound(kind, fields, r, errs):
    """bound(i) with per-point field bounds eb_f(i) = sum_l r_l(i) e_fl"""
    V, rho = _unpack(kind, fields)
    E = torch.tensor(np.stack(errs), dtype=torch.float64, device="cuda")      # (F, L+1)
    eb = E @ r                                                              # (F, N)
    shp = V[0].shape
    ebV = [eb[k].reshape(shp) for k in range(3)]
    return qoi_bound(kind, V, ebV, rho, eb[3].reshape(shp) if kind == "ke" else None)


def _sensitivity(kind, fields, r, errs, i):
    """d bound(i) / d eb_f at point i (central difference of the propagation rule)"""
    V, rho = _unpack(kind, fields)
    Vi = [v.reshape(-1)[i:i + 1] for v in V]
    ri = rho.reshape(-1)[i:i + 1] if kind == "ke" else None
    eb = [float(np.dot(e, r[:, i].cpu().numpy())) for e in errs]
    out = []
    for f in range(len(fields)):
        h = max(eb[f] * 1e-3, 1e-30)
        vals = []
        for s in (1.0, -1.0):
            e = list(eb)
            e[f] = max(e[f] + s * h, 0.0)
            t = [torch.tensor(x, dtype=torch.float64, device="cuda") for x in e]
            vals.append(float(qoi_bound(kind, Vi, t[:3], ri, t[3] if kind == "ke" else None)))
        out.append(max((vals[0] - vals[1]) / (2 * h), 0.0))
    return out


def guided_retrieve(kind, data, tau, rel, L, B=32, encoder="grouped", max_iter=8, batch=4, margin=0.97):
    """data as for halving_retrieve."""
    fields = [_Field(x, L, B, encoder) for x in data]
    shape = fields[0].shape
    r, off = level_influence(shape, L, data[0].dtype)
    # first pass: a coarse reconstruction (4x the reference's initial bounds)
    for f, x in zip(fields, data):
        f.retrieve_tolerance(value_range(x) * rel * 4)
    it, bound, met = 0, math.inf, False
    while it < max_iter:
        it += 1
        errs = [f.level_errors() for f in fields]
        est = _pointwise_bound(kind, fields, r, errs)
        bound = float(est.max())
        if bound <= tau:
            met = True
            break
        plan = [f.index.copy() for f in fields]
        target = tau * margin
        while True:
            i = int(torch.argmax(est))
            w_level = point_level_weights(shape, L, i, off, data[0].dtype)
            w_field = _sensitivity(kind, fields, r, [f.level_errors(p) for f, p in zip(fields, plan)], i)
            heap = []
            for fi, f in enumerate(fields):
                for l in range(L + 1):
                    b = plan[fi][l]
                    if b >= B:
                        continue
                    gain = w_field[fi] * w_level[l] * (f.errs[l, b] - f.errs[l, b + 1])
                    size = int(f.sizes[l, b])
                    eff = math.inf if size == 0 else gain / size
                    heapq.heappush(heap, (-eff, fi, l))
            if not heap:
                break
            for _ in range(batch):
                if not heap:
                    break
                _, fi, l = heapq.heappop(heap)
                plan[fi][l] += 1
            errs = [f.level_errors(p) for f, p in zip(fields, plan)]
            est = _pointwise_bound(kind, fields, r, errs)
            if float(est.max()) <= target:
                break
        for f, p in zip(fields, plan):
            f.retrieve_planes(p)
    return {"bytes": sum(f.bytes() for f in fields), "bound": bound, "met": met, "iterations": it,
            "achieved": _achieved(kind, fields, data), "index": [f.index.tolist() for f in fields]}
