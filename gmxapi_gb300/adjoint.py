"""Differentiable short-range nonbonded forces for force matching.

There is no counterpart in the reference, which only evaluates forces.  The
forward pass is the cluster-pair force/energy kernel (nblib
``ForceCalculator::compute``, api/nblib/gmxcalculator.cpp:88-101); the backward
pass is a hand-written CUDA kernel that walks the same pair list, recomputes
every pair term and returns, for upstream gradients G = dL/dF and
gE = dL/d(E_lj, E_coul):

* dL/dx  -- the Hessian-vector product with G plus the energy terms,
* dL/dq  -- per atom,
* dL/dnbfp -- per type pair, for the {6*C6, 12*C12} table (FP64 sums).

Per-type sigma/epsilon gradients follow by the chain rule through the
combination rule (``lorentz_berthelot_nbfp``), which autograd applies on the
ntypes x ntypes table.  Everything stays on the GPU and runs on the current
torch stream; there is no CPU path.
"""
from __future__ import annotations

import torch
from torch.autograd.function import once_differentiable

from .nblib import CoulombType, ForceCalculator, NBKernelOptions


class _LorentzBerthelot(torch.autograd.Function):
    """The combination rule on the GPU: one kernel forward, one kernel backward (float64)."""

    @staticmethod
    def forward(ctx, sigma, epsilon):
        from . import _lib

        nt = sigma.numel()
        table = torch.empty(nt, nt, 2, dtype=torch.float64, device=sigma.device)
        stream = torch.cuda.current_stream(sigma.device).cuda_stream
        code = _lib.load().nbx_lb_table_device(sigma.data_ptr(), epsilon.data_ptr(), nt, table.data_ptr(), stream)
        if code != 0:
            raise RuntimeError(f"nbx_lb_table_device failed ({code})")
        ctx.save_for_backward(sigma, epsilon)
        return table

    @staticmethod
    @once_differentiable
    def backward(ctx, g):
        from . import _lib

        sigma, epsilon = ctx.saved_tensors
        nt = sigma.numel()
        g = g.to(torch.float64).contiguous()
        gs = torch.empty_like(sigma)
        ge = torch.empty_like(epsilon)
        stream = torch.cuda.current_stream(sigma.device).cuda_stream
        code = _lib.load().nbx_lb_table_backward_device(sigma.data_ptr(), epsilon.data_ptr(), nt, g.data_ptr(),
                                                        gs.data_ptr(), ge.data_ptr(), stream)
        if code != 0:
            raise RuntimeError(f"nbx_lb_table_backward_device failed ({code})")
        return gs, ge


def lorentz_berthelot_nbfp(sigma: torch.Tensor, epsilon: torch.Tensor) -> torch.Tensor:
    """(ntypes, ntypes, 2) table {6*C6, 12*C12} from per-type sigma and epsilon.

    sigma_ij = (sigma_i + sigma_j) / 2, epsilon_ij = sqrt(epsilon_i epsilon_j),
    C6 = 4 eps s^6, C12 = 4 eps s^12 (the combination nblib applies in
    api/nblib/particletype.cpp and gmxsetup.cpp:143-166).  float64 CUDA vectors go through one
    kernel each way; other tensors (the FP64 reference on the CPU) through torch operations.  The
    table is symmetric by construction and is marked so (the engine then skips symmetrising it).
    """
    if sigma.is_cuda and sigma.dtype == torch.float64 and epsilon.dtype == torch.float64:
        table = _LorentzBerthelot.apply(sigma.contiguous(), epsilon.contiguous())
    else:
        sig = 0.5 * (sigma[:, None] + sigma[None, :])
        eps = torch.sqrt(epsilon[:, None] * epsilon[None, :])
        s6 = sig**6
        c6 = 4.0 * eps * s6
        c12 = c6 * s6
        table = torch.stack((6.0 * c6, 12.0 * c12), dim=-1)
    table._symmetric_types = True
    return table


class _ForceMatchingLoss(torch.autograd.Function):
    """sum_k (F_k - F_target_k)^2 as a float64 scalar; the same pass writes 2 (F - F_target)."""

    @staticmethod
    def forward(ctx, f, f_target):
        from . import _lib

        g = torch.empty_like(f)
        loss = torch.empty((), dtype=torch.float64, device=f.device)
        stream = torch.cuda.current_stream(f.device).cuda_stream
        code = _lib.load().nbx_match_loss_device(f.data_ptr(), f_target.data_ptr(), f.numel(), g.data_ptr(),
                                                 loss.data_ptr(), stream)
        if code != 0:
            raise RuntimeError(f"nbx_match_loss_device failed ({code})")
        ctx.save_for_backward(g)
        return loss

    @staticmethod
    @once_differentiable
    def backward(ctx, g_loss):
        (g,) = ctx.saved_tensors
        return g * g_loss, None


def force_matching_loss(f: torch.Tensor, f_target: torch.Tensor) -> torch.Tensor:
    """The force-matching loss sum |F - F_target|^2 (float64 scalar) of float32 CUDA forces.

    One kernel forward (the loss in FP64 and its gradient 2 (F - F_target) in the same pass) and
    one scaling kernel backward, in place of the three element-wise kernels each way that the torch
    expression ``((f - f_target) ** 2).sum()`` launches.  f_target is a constant (no gradient).
    """
    if not (f.is_cuda and f.dtype == torch.float32 and f_target.is_cuda and f_target.dtype == torch.float32):
        raise TypeError("force_matching_loss takes float32 CUDA tensors")
    if f.shape != f_target.shape:
        raise ValueError(f"shape mismatch: {tuple(f.shape)} vs {tuple(f_target.shape)}")
    return _ForceMatchingLoss.apply(f.contiguous(), f_target.detach().contiguous())


def static_list_options(rc: float = 0.9) -> NBKernelOptions:
    """Options for coordinates that do not move between searches (force matching on fixed
    frames, or a search on every call): the list radius equals the cut-off and the fresh
    list is pruned to cluster pairs with an atom pair inside rc, so no buffer pairs are
    computed."""
    return NBKernelOptions(coulomb_type=CoulombType.Pme, pairlist_cutoff=rc, rcoulomb=rc, rlist_inner=rc,
                           nstlist_prune=2)


class _NonbondedFunction(torch.autograd.Function):
    """(x, q, nbfp) -> (forces (N, 3) float32, energies [E_lj, E_coul] float64)."""

    @staticmethod
    def forward(ctx, x, q, nbfp, engine):
        calc = engine.calc
        calc.set_stream(torch.cuda.current_stream(x.device).cuda_stream)
        # the kernels read float32 parameters; the table gradient comes back in the
        # table's own dtype (FP64 sums when the table is float64)
        nbfp32 = nbfp.to(torch.float32).contiguous()
        engine._upload(q, nbfp32)
        f = torch.empty_like(x)
        e = torch.empty(2, dtype=torch.float64, device=x.device)  # written by the call, not added to
        calc.compute_device(x.data_ptr(), f.data_ptr(), e.data_ptr(), None)
        ctx.engine = engine
        ctx.save_for_backward(x, q, nbfp, nbfp32)
        # an unused output's gradient arrives as None instead of a zero-filled tensor
        ctx.set_materialize_grads(False)
        return f, e

    @staticmethod
    @once_differentiable
    def backward(ctx, g_f, g_e):
        x, q, nbfp, nbfp32 = ctx.saved_tensors
        calc = ctx.engine.calc
        dev = x.device
        calc.set_stream(torch.cuda.current_stream(dev).cuda_stream)
        # the handle may have seen other parameters since the forward pass (uploaded again then)
        ctx.engine._upload(q, nbfp32)
        g_f = torch.zeros_like(x) if g_f is None else g_f.to(torch.float32).contiguous()
        g_e = None if g_e is None else g_e.to(torch.float64).contiguous()
        need_x, need_q, need_p = ctx.needs_input_grad[:3]
        gx = torch.empty_like(x) if need_x else None
        gq = torch.empty_like(q) if need_q else None
        gp = torch.empty(nbfp.shape, dtype=torch.float64, device=dev) if need_p else None
        calc.backward_device(x.data_ptr(), g_f.data_ptr(), g_e.data_ptr() if g_e is not None else None,
                             gx.data_ptr() if gx is not None else None, gq.data_ptr() if gq is not None else None,
                             gp.data_ptr() if gp is not None else None)
        return gx, gq, (gp.to(nbfp.dtype) if gp is not None else None), None


class DifferentiableNonbonded:
    """Pair-list force field on one GPU whose forces and energies are differentiable.

    ``engine(x, q, nbfp)`` returns ``(forces, energies)`` for coordinates
    ``x`` (N, 3) float32, charges ``q`` (N,) float32 and the type table
    ``nbfp`` (ntypes, ntypes, 2) float32 or float64, all CUDA tensors.  ``nbfp`` is
    symmetrised before use so its gradient does not depend on which atom of a
    pair the list puts in the i-cluster.  The pair list is rebuilt from ``x``
    on every call unless ``search=False`` (then the list of the last search
    is used); the default options list exactly the pairs within the cut-off
    (``static_list_options``), so with moving coordinates and ``search=False``
    pass options with a buffer (rlist > rc).
    """

    def __init__(self, system, options: NBKernelOptions | None = None, device: int = 0):
        opts = options or static_list_options()
        opts.compute_virial_and_energy = True
        self.system = system
        self.ntypes = int(system.ntypes)
        self.device = torch.device("cuda", device)
        self.calc = ForceCalculator(system, opts, device)
        self._uploaded = None

    def _upload(self, q: torch.Tensor, nbfp32: torch.Tensor):
        """Charges and float32 type table to the handle, unless the same storage, unmodified, was
        the last one uploaded.  The uploaded tensors are kept referenced, so their memory cannot be
        reused by another tensor while their addresses serve as the key."""
        key = (q.data_ptr(), q._version, nbfp32.data_ptr(), nbfp32._version)
        if self._uploaded is None or key != self._uploaded[0]:
            self.calc.set_parameters_device(q.data_ptr(), nbfp32.data_ptr())
            self._uploaded = (key, q, nbfp32)

    def search(self, x: torch.Tensor):
        self.calc.set_stream(torch.cuda.current_stream(x.device).cuda_stream)
        self.calc.search_device(x.detach().contiguous().data_ptr())

    def __call__(self, x: torch.Tensor, q: torch.Tensor, nbfp: torch.Tensor, search: bool = True):
        if not (x.is_cuda and q.is_cuda and nbfp.is_cuda):
            raise ValueError("x, q and nbfp must be CUDA tensors (there is no CPU path)")
        nt = self.ntypes
        if x.shape != (self.system.n, 3) or q.shape != (self.system.n,) or nbfp.shape != (nt, nt, 2):
            raise ValueError("x must be (N, 3), q (N,) and nbfp (ntypes, ntypes, 2)")
        x = x.to(torch.float32).contiguous()
        q = q.to(torch.float32).contiguous()
        if not getattr(nbfp, "_symmetric_types", False):
            nbfp = (0.5 * (nbfp + nbfp.transpose(0, 1))).contiguous()
        if search:
            self.search(x)
        return _NonbondedFunction.apply(x, q, nbfp, self)

    def close(self):
        self.calc.close()


class _TypeScaledCharges(torch.autograd.Function):
    @staticmethod
    def forward(ctx, scale, helper):
        ctx.helper = helper
        return (helper.q0 * scale[helper.types]).to(torch.float32)

    @staticmethod
    @once_differentiable
    def backward(ctx, g):
        h = ctx.helper
        # per-type sums of q0 * dL/dq over the type-sorted atoms: prefix sums, no atomics
        v = (h.q0 * g.to(h.q0.dtype))[h.perm]
        cs = torch.cat([v.new_zeros(1), torch.cumsum(v, 0)])
        return cs[h.ends] - cs[h.starts], None


class TypeScaledCharges:
    """q_i = q0_i * scale[type_i] with a cheap backward (dL/dscale by prefix sums over the
    atoms sorted by type, instead of a scatter of N values onto a few addresses)."""

    def __init__(self, q0: torch.Tensor, types: torch.Tensor, ntypes: int):
        self.q0 = q0.to(torch.float64)
        self.types = types.to(torch.long)
        self.perm = torch.argsort(self.types, stable=True)
        counts = torch.bincount(self.types, minlength=ntypes)
        self.ends = torch.cumsum(counts, 0)
        self.starts = self.ends - counts

    def __call__(self, scale: torch.Tensor) -> torch.Tensor:
        return _TypeScaledCharges.apply(scale, self)


class _BatchMatchLoss(torch.autograd.Function):
    """(q, nbfp) -> force-matching loss of a batch; one graph launch computes the loss and
    both gradients, which backward returns scaled by the upstream gradient."""

    @staticmethod
    def forward(ctx, q, nbfp, matcher):
        loss = matcher._run(q, nbfp)
        ctx.matcher = matcher
        ctx.nbfp_dtype = nbfp.dtype
        return loss

    @staticmethod
    @once_differentiable
    def backward(ctx, g):
        m = ctx.matcher
        return g.to(torch.float32) * m._gq, (g * m._gnbfp).to(ctx.nbfp_dtype), None


class BatchForceMatcher:
    """Force matching over a batch of systems with shared type parameters.

    ``matcher(q, nbfp)`` returns the loss sum over systems and atoms of
    |F - F_target|^2 (FP64) as a differentiable scalar: q holds all systems'
    charges (concatenated atom order, float32) and nbfp the shared
    (ntypes, ntypes, 2) table.  Each call is one CUDA-graph launch on the GPU
    (parameters -> forces, energies, virials -> loss -> adjoint); the pair
    lists are built once from the fixed coordinates.
    """

    def __init__(self, systems, f_target: torch.Tensor, options: NBKernelOptions | None = None, device: int = 0):
        from .batch import BatchForceCalculator

        opts = options or static_list_options()
        opts.compute_virial_and_energy = True
        self.dev = torch.device("cuda", device)
        self.batch = BatchForceCalculator(systems, opts, device)
        self.nsys = len(systems)
        self.ntypes = int(systems[0].ntypes)
        self.x = torch.cat([torch.as_tensor(s.x, dtype=torch.float32).reshape(-1) for s in systems]).to(self.dev)
        n = self.x.numel() // 3
        self.f_target = f_target.to(self.dev, torch.float32).reshape(-1).contiguous()
        if self.f_target.numel() != 3 * n:
            raise ValueError("f_target must hold 3 values per atom of the batch")
        self.batch.set_stream(torch.cuda.current_stream(self.dev).cuda_stream)
        self.batch.search_device(self.x.data_ptr())
        self._loss = torch.zeros(1, dtype=torch.float64, device=self.dev)
        self._gq = torch.empty(n, dtype=torch.float32, device=self.dev)
        self._gnbfp = torch.empty(self.ntypes, self.ntypes, 2, dtype=torch.float64, device=self.dev)
        self.energies = torch.zeros(2 * self.nsys, dtype=torch.float64, device=self.dev)
        self.virials = torch.zeros(9 * self.nsys, dtype=torch.float64, device=self.dev)
        self._q = torch.empty(n, dtype=torch.float32, device=self.dev)
        self._nbfp = torch.empty(self.ntypes * self.ntypes * 2, dtype=torch.float32, device=self.dev)

    def _run(self, q, nbfp):
        # fixed buffers keep the captured graph's pointers valid between calls
        self._q.copy_(q.detach().reshape(-1))
        self._nbfp.copy_((0.5 * (nbfp + nbfp.transpose(0, 1))).detach().reshape(-1))
        self.batch.set_stream(torch.cuda.current_stream(self.dev).cuda_stream)
        self.batch.force_match_device(self.x.data_ptr(), self._q.data_ptr(), self._nbfp.data_ptr(),
                                      self.f_target.data_ptr(), self._loss.data_ptr(), self._gq.data_ptr(),
                                      self._gnbfp.data_ptr(), self.energies.data_ptr(), self.virials.data_ptr())
        # the table gradient of the symmetrised table, back onto the input table
        self._gnbfp.copy_(0.5 * (self._gnbfp + self._gnbfp.transpose(0, 1)))
        return self._loss[0].clone()

    def __call__(self, q: torch.Tensor, nbfp: torch.Tensor):
        return _BatchMatchLoss.apply(q, nbfp, self)

    def close(self):
        self.batch.close()
