"""The learned warm start, driven from Python: training-set generation with
the library's own solver, training with the library's own BF16 tensor-core
forward/backward kernels and Adam, and the warm-started solve.

Torch is used only for device buffers, shuffling indices and gathering
mini-batches; every network evaluation and update runs in libmsfem_gpu.so.
"""
import ctypes
import time

import numpy as np

from . import _abi, workloads

NODES = 33 * 33


class Surrogate:
    """msfem_surrogate handle (a network on the engine's device)."""

    def __init__(self, engine, seed=1234):
        self.engine = engine
        self.lib = engine.lib
        h = ctypes.c_void_p()
        rc = self.lib.msfem_surrogate_create(engine.handle, seed, ctypes.byref(h))
        if rc != _abi.OK:
            raise _abi.MsfemError(rc, _abi.last_error(self.lib))
        self.handle = h
        self.n_params = int(self.lib.msfem_surrogate_param_count())

    def close(self):
        if self.handle:
            self.lib.msfem_surrogate_destroy(self.handle)
            self.handle = None

    def _check(self, rc):
        if rc != _abi.OK:
            raise _abi.MsfemError(rc, _abi.last_error(self.lib))

    def get_params(self):
        out = np.zeros(self.n_params, dtype=np.float32)
        self._check(self.lib.msfem_surrogate_get_params(self.handle, out.ctypes.data))
        return out

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        assert p.size == self.n_params
        self._check(self.lib.msfem_surrogate_set_params(self.handle, p.ctypes.data))

    def predict(self, feats, out):
        self._check(self.lib.msfem_surrogate_predict(self.handle, feats.data_ptr(), feats.shape[0],
                                                     out.data_ptr()))

    def gradients(self, feats, targets):
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = ctypes.c_double()
        self._check(self.lib.msfem_surrogate_gradients(self.handle, feats.data_ptr(), targets.data_ptr(),
                                                       feats.shape[0], g.ctypes.data, ctypes.byref(loss)))
        return loss.value, g

    def train_step(self, feats, targets, lr, want_loss=True):
        """One Adam step; returns the batch loss, or None without want_loss
        (no device synchronisation: the step's launches queue behind the
        previous ones)."""
        loss = ctypes.c_double()
        self._check(self.lib.msfem_surrogate_train_step(self.handle, feats.data_ptr(), targets.data_ptr(),
                                                        feats.shape[0], lr,
                                                        ctypes.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def attach(self):
        self._check(self.lib.msfem_attach_surrogate(self.engine.handle, self.handle))

    def detach(self):
        self._check(self.lib.msfem_attach_surrogate(self.engine.handle, None))


def device_problem(engine, prob, torch):
    """Corners and the GPU-tabulated coefficient of a 2D N = 32 problem in
    device memory; returns (desc, keep) with desc in DEVICE memory mode."""
    n = prob["corners"].shape[0]
    corners = torch.from_numpy(np.ascontiguousarray(prob["corners"])).cuda()
    c = prob["coef"]
    dt = _abi.BatchDesc()
    dt.dim, dt.n_cells, dt.n_fine = 2, n, 32
    dt.corners = corners.data_ptr()
    dt.coef.kind = c["kind"]
    for i, v in enumerate(c.get("params", [])):
        dt.coef.params[i] = float(v)
    keep = [corners]
    if c.get("modes") is not None:
        modes = torch.from_numpy(np.ascontiguousarray(c["modes"])).cuda()
        keep.append(modes)
        dt.coef.modes = modes.data_ptr()
        dt.coef.n_modes = modes.shape[1]
    dt.memory = _abi.MEM_DEVICE
    dt.tol, dt.maxit = 1e-10, 1000
    size = engine.lib.msfem_tabulated_size(ctypes.byref(dt), 3)
    tab = torch.empty(size, dtype=torch.float64, device="cuda")
    rc = engine.lib.msfem_tabulate_coefficient(engine.handle, ctypes.byref(dt), 3, tab.data_ptr())
    if rc != _abi.OK:
        raise _abi.MsfemError(rc, _abi.last_error(engine.lib))
    keep.append(tab)
    d = _abi.BatchDesc()
    d.dim, d.n_cells, d.n_fine = 2, n, 32
    d.corners = corners.data_ptr()
    d.coef.kind = _abi.COEF_TABULATED
    d.coef.ncomp = 3
    d.coef.qp_values = tab.data_ptr()
    d.f_value = float(prob.get("f_value", 1.0))
    d.tol, d.maxit = 1e-10, 1000
    d.memory = _abi.MEM_DEVICE
    return d, keep


def features(engine, desc, torch):
    out = torch.empty((desc.n_cells, 3, 33, 33), dtype=torch.float32, device="cuda")
    rc = engine.lib.msfem_surrogate_features(engine.handle, ctypes.byref(desc), out.data_ptr())
    if rc != _abi.OK:
        raise _abi.MsfemError(rc, _abi.last_error(engine.lib))
    return out


def solve_device(engine, desc, torch, precision=_abi.PREC_MIXED, want_basis=False, warm=_abi.WARM_NONE,
                 tol=1e-10):
    """Device-resident batch solve; returns dict with M, iters, basis (torch) and stats."""
    n = desc.n_cells
    desc.precision = precision
    desc.warm_start = warm
    desc.tol = tol
    M = torch.empty((n, 4, 4), dtype=torch.float64, device="cuda")
    F = torch.empty((n, 4), dtype=torch.float64, device="cuda")
    st = torch.empty(n, dtype=torch.int32, device="cuda")
    it = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    basis = torch.empty((n, 4, NODES), dtype=torch.float64, device="cuda") if want_basis else None
    rc, stats = engine.run_desc(desc, M.data_ptr(), F.data_ptr(), basis.data_ptr() if want_basis else None,
                                st.data_ptr(), it.data_ptr(), stats=True)
    desc.warm_start = _abi.WARM_NONE
    return {"M": M, "F": F, "status": st, "iters": it, "basis": basis, "stats": stats, "rc": rc}


def training_set(engine, torch, seeds=None, K=64, log=None):
    """Basis solves of random-Fourier tensor fields (the fourier_square family with
    new seeds): features and targets delta = phi - Q1 on the device."""
    seeds = seeds or [(100 + 7 * i, 1000 + 7 * i, 10000 + 7 * i) for i in range(12)]
    feats, tgts = [], []
    for sd in seeds:
        t0 = time.time()
        prob = workloads.fourier_square(K=K, N=32, seeds=sd)
        desc, keep = device_problem(engine, prob, torch)
        res = solve_device(engine, desc, torch, want_basis=True)
        assert res["stats"]["cells_failed"] == 0
        f = features(engine, desc, torch)
        delta = torch.empty((desc.n_cells, 4, 33, 33), dtype=torch.float32, device="cuda")
        rc = engine.lib.msfem_surrogate_targets(engine.handle, res["basis"].data_ptr(), desc.n_cells,
                                                delta.data_ptr())
        if rc != _abi.OK:
            raise _abi.MsfemError(rc, _abi.last_error(engine.lib))
        feats.append(f)
        tgts.append(delta)
        del keep, res
        if log:
            log(f"training fields {sd}: {desc.n_cells} cells in {time.time() - t0:.2f} s")
    return torch.cat(feats), torch.cat(tgts)


def library_stream(torch):
    """cudaStream_t handle of torch's current stream, for msfem_set_stream.
    torch reports its legacy default stream as 0, and a NULL stream would put
    the library on the handle's own non-blocking stream, which does not wait
    for work on the legacy stream: map 0 to cudaStreamLegacy."""
    h = torch.cuda.current_stream().cuda_stream
    return h if h else _abi.CUDA_STREAM_LEGACY


def train(sur, feats, targets, torch, epochs=20, batch=256, lr=1e-3, seed=0, log=None, loss_every=1):
    """Adam with a fixed learning rate over shuffled mini-batches.  The batch
    loss is read back (a device synchronisation) every `loss_every` steps and
    at the last step of each epoch; an epoch's history entry is the mean of
    the losses read in it (every step's by default)."""
    n = feats.shape[0]
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    steps = max(1, (n - batch) // batch + 1) if n >= batch else 0
    # the mini-batch gathers run on torch's stream and the steps must follow
    # them (and torch may reuse a batch's memory only after its step): the
    # library launches on torch's current stream while training
    engine = sur.engine
    prev = getattr(engine, "stream_handle", 0)
    engine.set_stream(library_stream(torch))
    try:
        history = _train_epochs(sur, feats, targets, torch, epochs, batch, lr, gen, n, steps, loss_every, log)
    finally:
        engine.set_stream(prev)
    return history


def _train_epochs(sur, feats, targets, torch, epochs, batch, lr, gen, n, steps, loss_every, log):
    history = []
    t0 = time.time()
    for ep in range(epochs):
        perm = torch.randperm(n, device="cuda", generator=gen)
        tot, cnt = 0.0, 0
        for k, b0 in enumerate(range(0, n - batch + 1, batch)):
            idx = perm[b0:b0 + batch]
            fb = feats.index_select(0, idx).contiguous()
            tb = targets.index_select(0, idx).contiguous()
            read = (k % loss_every == loss_every - 1) or k == steps - 1
            loss = sur.train_step(fb, tb, lr, want_loss=read)
            if read:
                tot += loss
                cnt += 1
        history.append(tot / max(1, cnt))
        if log:
            log(f"epoch {ep + 1}: loss {history[-1]:.3e} ({time.time() - t0:.1f} s)")
    return history
