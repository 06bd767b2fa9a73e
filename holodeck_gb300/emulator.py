"""Learned emulator of SAM libraries: an ensemble of MLPs that maps the parameters of a library's
parameter space to per-frequency statistics of the characteristic strain, trained on libraries the
GPU SAM writes (:func:`holodeck_gb300.librarian.batch.run_library`).

No reference counterpart: the reference emulates libraries with Gaussian processes
(holodeck/gps/gp_utils.py), fitted to the library's spectra after the fact.  Here the network is a
drop-in answer to "what does the SAM give at these parameters", and the plain GPU SAM stays its
fallback and its judge: a query outside the parameter box the network was trained on, or one on which
the ensemble members disagree by more than ``max_spread`` dex, is re-solved exactly.

Statistics per frequency (the network's outputs, ``nfreqs * 4`` of them, frequency-major):
the 5th, 50th and 95th percentiles over realizations of log10 hc, with hc^2 = hc_bg^2 + sum of the
loudest sources' hc_ss^2 (the total characteristic strain of a realization), and the median over
realizations of log10 of the loudest source's hc.

Network: inputs are the parameters mapped to [-1, 1] over the space's extrema and zero-padded to 16;
``depth`` hidden layers of ``width`` with SiLU; a linear output layer; targets standardised per output.
Forward, backward and AdamW run in the hand-written tensor-core kernels of ``csrc/hgb_mlp.cu``
(bf16 weights and activations, fp32 accumulation and master weights); PyTorch only holds the buffers.
"""

import ctypes
import math
import time

import numpy as np

from . import _device as D
from . import _native as N

STATS = ("log10_hc_p05", "log10_hc_p50", "log10_hc_p95", "log10_hc_loudest_p50")
INPUT_PAD = 16
HIDDEN_STRIDE = 256
LOG10_FLOOR = -40.0


def bf16_bits(x):
    """bfloat16 bit patterns (uint16) of values rounded to the nearest bfloat16, ties to even: the
    conversion the device makes, done on the host for the graphed query path's pinned inputs."""
    bits = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    return ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype(np.uint16)


def strain_statistics(hc_ss, hc_bg):
    """(F, 4) statistics of one model evaluation from hc_ss (F, R, L) and hc_bg (F, R) (see module)."""
    hc_ss = np.asarray(hc_ss, dtype=np.float64)
    hc_bg = np.asarray(hc_bg, dtype=np.float64)
    hc2 = hc_bg ** 2 + (hc_ss ** 2).sum(axis=-1)
    with np.errstate(divide="ignore"):
        lg = np.maximum(0.5 * np.log10(hc2), LOG10_FLOOR)
        loud = np.maximum(np.log10(hc_ss[..., 0]), LOG10_FLOOR)
    p = np.percentile(lg, [5.0, 50.0, 95.0], axis=1)
    return np.stack([p[0], p[1], p[2], np.median(loud, axis=1)], axis=-1)


class MLPEnsemble:
    """E independently initialised MLPs with the layer widths ``dims`` (each a multiple of 16 in
    [16, 256]), trained together: every step feeds all members the same batch."""

    def __init__(self, dims, members=4, seed=0, device=None):
        t = D.torch()
        self.dims = [int(d) for d in dims]
        if len(self.dims) - 1 > N.MLP_MAX_LAYERS:
            raise ValueError(f"at most {N.MLP_MAX_LAYERS} layers")
        if any(d % 16 or not 16 <= d <= 256 for d in self.dims):
            raise ValueError(f"layer widths must be multiples of 16 in [16, 256]: {self.dims}")
        self.members = int(members)
        self.device = D.device(device)
        self.L = len(self.dims) - 1
        self.struct = N.HgbMlp()
        self.struct.n_layers = self.L
        self.struct.n_members = self.members
        for ii, d in enumerate(self.dims):
            self.struct.dims[ii] = d
        lib = N.load()
        self.n_params = int(lib.hgb_mlp_param_count(ctypes.byref(self.struct)))
        self.n_weights = int(lib.hgb_mlp_weight_count(ctypes.byref(self.struct)))
        self.params = t.as_tensor(self.initial_params(seed), device=self.device)
        self.weights = t.empty((self.members, self.n_weights), dtype=t.bfloat16, device=self.device)
        self.m1 = t.zeros_like(self.params)
        self.m2 = t.zeros_like(self.params)
        self.grad = t.zeros_like(self.params)
        self.step_count = 0
        self._bind()
        N.call("hgb_mlp_pack_weights", ctypes.byref(self.struct), N.ptr(self.params), N.ptr(self.weights),
               N.stream_handle())
        self._buffers = {}
        self.status = D.StatusWord(self.device)

    def initial_params(self, seed):
        """fp32 [E, P]: uniform(+-sqrt(3 / fan_in)) weights (unit-variance pre-activations for
        unit-variance inputs), output layer scaled by 0.1, zero biases; member m seeded (seed, m)."""
        out = np.zeros((self.members, self.n_params), dtype=np.float32)
        for m in range(self.members):
            rng = np.random.default_rng([int(seed), m])
            off = 0
            for ll in range(self.L):
                k, n = self.dims[ll], self.dims[ll + 1]
                a = math.sqrt(3.0 / k) * (0.1 if ll == self.L - 1 else 1.0)
                w = rng.uniform(-a, a, size=(n, k)).astype(np.float32)
                out[m, off:off + n * k] = w.ravel()
                off += n * k + n
        return out

    def layer(self, params, member, ll):
        """(W [N][K], b [N]) of one member and layer from a [E, P] host array."""
        off = 0
        for jj in range(ll):
            off += self.dims[jj + 1] * self.dims[jj] + self.dims[jj + 1]
        k, n = self.dims[ll], self.dims[ll + 1]
        row = params[member]
        return row[off:off + n * k].reshape(n, k), row[off + n * k:off + n * k + n]

    def _bind(self):
        self.struct.params = self.params.data_ptr()
        self.struct.weights = self.weights.data_ptr()

    def _buffers_for(self, batch, train, owner=None):
        key = (int(batch), bool(train), owner)
        buf = self._buffers.get(key)
        if buf is None:
            t = D.torch()
            hid = max(self.L - 1, 1) * self.members * batch * HIDDEN_STRIDE
            buf = dict(act=t.empty(hid, dtype=t.bfloat16, device=self.device),
                       pre=t.empty(hid, dtype=t.float32, device=self.device) if train else None,
                       out=t.empty((self.members, batch, self.dims[-1]), dtype=t.float32, device=self.device))
            if train:
                ws = N.load().hgb_mlp_backward_workspace_bytes(ctypes.byref(self.struct), int(batch))
                buf["ws"] = D.workspace(ws, self.device)
                buf["ws_bytes"] = int(ws)
                buf["loss"] = t.empty(self.members, dtype=t.float32, device=self.device)
            self._buffers[key] = buf
        return buf

    def forward(self, x, train=False, member_stride=0, owner=None):
        """Outputs [E, B, n_out] (fp32) for bf16 inputs x [B, dims[0]] (one batch for all members).
        The activation buffers are per (batch, train, owner): a captured graph passes its own owner
        so that eager calls never write into the buffers its replays read."""
        t = D.torch()
        assert x.dtype == t.bfloat16 and x.is_contiguous() and x.shape[-1] == self.dims[0]
        batch = int(x.shape[-2])
        buf = self._buffers_for(batch, train, owner)
        N.call("hgb_mlp_forward", ctypes.byref(self.struct), N.ptr(x), int(member_stride), batch, N.ptr(buf["act"]),
               N.ptr(buf["pre"]), N.ptr(buf["out"]), self.status.ptr, N.stream_handle())
        N.add_launches(self.L)
        return buf["out"]

    def forward_fused(self, x, member_stride=0, owner=None):
        """:meth:`forward` (inference) for at most ``_native.MLP_FUSED_MAX_BATCH`` rows in one launch
        (hgb_mlp_forward_fused: weights and activations on chip, CUDA-core products).  The fp32 sums
        run in another order than the tensor-core path's, so an activation can round to the
        neighbouring bf16 value."""
        t = D.torch()
        assert x.dtype == t.bfloat16 and x.is_contiguous() and x.shape[-1] == self.dims[0]
        batch = int(x.shape[-2])
        if batch > N.MLP_FUSED_MAX_BATCH:
            raise ValueError(f"the fused forward takes at most {N.MLP_FUSED_MAX_BATCH} rows, got {batch}")
        buf = self._buffers_for(batch, False, ("fused", owner))
        N.call("hgb_mlp_forward_fused", ctypes.byref(self.struct), N.ptr(x), int(member_stride), batch,
               N.ptr(buf["out"]), self.status.ptr, N.stream_handle())
        return buf["out"]

    def gradients(self, x, target):
        """Forward + backward of one batch: loss [E] (device) and self.grad [E, P]."""
        batch = int(x.shape[-2])
        out = self.forward(x, train=True)
        buf = self._buffers[(batch, True, None)]
        N.call("hgb_mlp_backward", ctypes.byref(self.struct), N.ptr(x), 0, batch, N.ptr(buf["act"]),
               N.ptr(buf["pre"]), N.ptr(out), N.ptr(target), 0, N.ptr(self.grad), N.ptr(buf["loss"]),
               N.ptr(buf["ws"]), buf["ws_bytes"], self.status.ptr, N.stream_handle())
        N.add_launches(2 * self.L + 1)
        return buf["loss"]

    def train_step(self, x, target, lr, weight_decay=1e-4, beta1=0.9, beta2=0.999, eps=1e-8):
        loss = self.gradients(x, target)
        self.step_count += 1
        N.call("hgb_mlp_adamw", ctypes.byref(self.struct), N.ptr(self.params), N.ptr(self.grad), N.ptr(self.m1),
               N.ptr(self.m2), N.ptr(self.weights), self.step_count, float(lr), float(beta1), float(beta2),
               float(eps), float(weight_decay), N.stream_handle())
        return loss

    def check_status(self, code=None):
        """Raise if a kernel since the last check gave up waiting for the tensor core (its outputs
        were not written).  The status word is cleared first, so one timeout does not fail later
        calls.  ``code``: a status value already read (the graphed path copies it to the host)."""
        if code is None:
            code = self.status.read()
            if code:
                self.status.reset()
        if code & N.STATUS_ITERATION_LIMIT:
            raise N.NativeError("an MLP kernel timed out waiting for the tensor core; its outputs are not valid")

    def state(self):
        return dict(dims=np.array(self.dims), members=self.members, params=D.to_host(self.params))

    def load_params(self, params):
        t = D.torch()
        self.params.copy_(t.as_tensor(np.asarray(params, dtype=np.float32), device=self.device))
        N.call("hgb_mlp_pack_weights", ctypes.byref(self.struct), N.ptr(self.params), N.ptr(self.weights),
               N.stream_handle())


class Emulator:
    """Ensemble emulator of a parameter space's library statistics (see the module docstring)."""

    def __init__(self, space, nfreqs=40, members=4, width=256, depth=4, seed=0, device=None):
        ext = np.asarray(space.extrema, dtype=np.float64)
        self.lo, self.hi = ext[:, 0], ext[:, 1]
        self.param_names = list(space.param_names)
        self.nfreqs = int(nfreqs)
        self.n_out = 4 * self.nfreqs
        self.n_pad = -(-self.n_out // 16) * 16     # output layer width: padded columns are trained to 0
        dims = [INPUT_PAD] + [int(width)] * int(depth) + [self.n_pad]
        self.net = MLPEnsemble(dims, members=members, seed=seed, device=device)
        self.mu = np.zeros(self.n_out)
        self.sd = np.ones(self.n_out)
        self.residual_scatter = None   # per-output training-residual scatter (dex), set by fit()
        self._graphs = {}

    # ---- data

    def unit(self, params):
        """Parameters (Q, P) -> coordinates in the training box, [0, 1] inside."""
        return (np.atleast_2d(np.asarray(params, dtype=np.float64)) - self.lo) / (self.hi - self.lo)

    def inputs(self, params):
        """bf16 device inputs (Q, 16): box coordinates mapped to [-1, 1], zero-padded."""
        t = D.torch()
        u = self.unit(params)
        x = np.zeros((u.shape[0], INPUT_PAD), dtype=np.float32)
        x[:, :u.shape[1]] = 2.0 * u - 1.0
        return t.as_tensor(x, device=self.net.device).to(t.bfloat16)

    # ---- training

    def fit(self, params, stats, epochs=300, batch=512, lr=2e-3, weight_decay=1e-4, warmup=0.03, seed=0,
            log=None):
        """Train on library samples: params (S, P), stats (S, F, 4).  Cosine learning-rate schedule
        with linear warm-up; returns the per-epoch mean training loss (standardised units)."""
        t = D.torch()
        y = np.asarray(stats, dtype=np.float64).reshape(len(stats), self.n_out)
        self.mu = y.mean(axis=0)
        self.sd = np.maximum(y.std(axis=0), 1e-6)
        x_all = self.inputs(params)
        ys = np.zeros((len(y), self.n_pad), dtype=np.float32)
        ys[:, :self.n_out] = (y - self.mu) / self.sd
        y_all = t.as_tensor(ys, device=self.net.device)
        ns = x_all.shape[0]
        batch = min(int(batch), ns)
        steps_per_epoch = ns // batch
        total = max(1, epochs * steps_per_epoch)
        rng = np.random.default_rng(seed)
        history = []
        step = 0
        for ep in range(epochs):
            perm = t.as_tensor(rng.permutation(ns), device=self.net.device)
            losses = []
            for ii in range(steps_per_epoch):
                idx = perm[ii * batch:(ii + 1) * batch]
                frac = step / total
                rate = lr * min(1.0, frac / max(warmup, 1e-9)) * 0.5 * (1.0 + math.cos(math.pi * frac))
                loss = self.net.train_step(x_all.index_select(0, idx).contiguous(),
                                           y_all.index_select(0, idx).contiguous(), max(rate, lr * 1e-3),
                                           weight_decay=weight_decay)
                losses.append(loss)
                step += 1
            history.append(float(t.stack(losses).mean().item()))
            if log is not None and (ep % max(1, epochs // 10) == 0 or ep == epochs - 1):
                log(f"epoch {ep}: loss {history[-1]:.5f}")
        self.net.check_status()
        self.residual_scatter = self._training_residual_scatter(x_all, y)
        return history

    def _training_residual_scatter(self, x_all, y, chunk=4096):
        """Per output (n_out,), in dex: the standard deviation over the training samples of the
        ensemble mean's residual, i.e. the emulator's typical error on its own library (the
        realization noise of the library's statistics plus the fit's error, whose heavy tail makes it
        larger than the noise alone).  :meth:`predict` can scale each output's spread by it."""
        t = D.torch()
        res = []
        for i0 in range(0, x_all.shape[0], chunk):
            out = self.net.forward(x_all[i0:i0 + chunk].contiguous())
            res.append(D.to_host(out.mean(dim=0))[:, :self.n_out].astype(np.float64))
        self.net.check_status()
        pred = np.concatenate(res) * self.sd + self.mu
        return np.std(pred - y, axis=0)

    # ---- queries

    def predict_members(self, params):
        """Per-member statistics (E, Q, F, 4) in log10 units."""
        out = D.to_host(self.net.forward(self.inputs(params)))[..., :self.n_out].astype(np.float64)
        self.net.check_status()
        out = out * self.sd + self.mu
        return out.reshape(out.shape[0], out.shape[1], self.nfreqs, 4)

    def predict(self, params, spread_stats=None, residual_scaled=False, max_spread=0.05):
        """(mean (Q, F, 4), spread (Q,), inside (Q,)): the ensemble mean, the largest standard
        deviation over members (dex) of the statistics named in ``spread_stats`` (default: all of
        :data:`STATS`) at any frequency, and whether the query lies in the training box.

        ``residual_scaled``: each output's standard deviation is first divided by its threshold
        max(``max_spread``, the output's training-residual scatter, see :meth:`fit`) and the largest
        ratio times ``max_spread`` is returned, so that ``spread > max_spread`` flags a query whose
        members disagree by more than both ``max_spread`` and the emulator's typical error on that
        output over its training library."""
        mem = self.predict_members(params)
        u = self.unit(params)
        inside = np.all((u >= 0.0) & (u <= 1.0), axis=1)
        cols = list(range(4)) if spread_stats is None else [STATS.index(nm) for nm in spread_stats]
        std = mem.std(axis=0)
        if residual_scaled:
            if getattr(self, "residual_scatter", None) is None:
                raise ValueError("residual_scaled needs the residual scatter that fit() records")
            thr = np.maximum(max_spread, self.residual_scatter.reshape(self.nfreqs, 4))
            std = std / thr[None] * max_spread
        return mem.mean(axis=0), std[..., cols].max(axis=(1, 2)), inside

    def query(self, params, fallback=None, max_spread=0.05, spread_stats=None, residual_scaled=False):
        """Statistics (Q, F, 4) with the plain SAM as fallback: queries outside the training box or
        with ensemble spread (of ``spread_stats``, optionally residual-scaled, see :meth:`predict`)
        above ``max_spread`` dex are re-solved by ``fallback(param_row) -> (F, 4)`` (e.g.
        :func:`sam_fallback`).  Returns (stats, solved_by_sam mask).  If the network's kernels fail
        (a tensor-core wait gave up), every query is re-solved by ``fallback``; without one the
        error is raised."""
        try:
            mean, spread, inside = self.predict(params, spread_stats=spread_stats, residual_scaled=residual_scaled,
                                                max_spread=max_spread)
            redo = (~inside) | (spread > max_spread)
        except N.NativeError:
            if fallback is None:
                raise
            nq = np.atleast_2d(params).shape[0]
            mean = np.full((nq, self.nfreqs, 4), np.nan)
            redo = np.ones(nq, dtype=bool)
        if fallback is not None:
            for qq in np.flatnonzero(redo):
                mean[qq] = fallback(np.atleast_2d(params)[qq])
        return mean, redo

    def graphed(self, batch, fused=None):
        """A CUDA-graph query path for batches of ``batch`` parameter rows: the host-to-device copy of
        the inputs, the network (the fused one-launch forward up to ``_native.MLP_FUSED_MAX_BATCH``
        rows, the tensor-core layers above) and the device-to-host copy of the outputs replay as one
        graph launch.  Returns a callable params (Q <= batch, P) -> ensemble-mean statistics (Q, F, 4).
        ``fused``: force (True) or exclude (False) the fused forward; None picks by batch."""
        use_fused = (batch <= N.MLP_FUSED_MAX_BATCH) if fused is None else bool(fused)
        key = (int(batch), use_fused)
        g = self._graphs.get(key)
        if g is None:
            g = _GraphedForward(self, batch, use_fused)
            self._graphs[key] = g
        return g

    def native(self, batch=1):
        """The lowest-latency query path for up to ``batch`` (<= ``_native.MLP_FUSED_MAX_BATCH``) rows:
        one call of ``hgb_emulator_query``, which maps the parameters into the box, rounds them to
        bf16 in pinned memory, runs the fused forward on the current stream, synchronises and forms
        the scaled ensemble mean on the host thread.  Returns a callable params (Q <= batch, P) ->
        ensemble-mean statistics (Q, F, 4); it raises NativeError if the kernel's bounded wait gave up."""
        key = ("native", int(batch))
        q = self._graphs.get(key)
        if q is None:
            q = _NativeQuery(self, batch)
            self._graphs[key] = q
        return q

    def state(self):
        rs = getattr(self, "residual_scatter", None)
        extra = {} if rs is None else dict(residual_scatter=rs)
        return dict(lo=self.lo, hi=self.hi, mu=self.mu, sd=self.sd, nfreqs=self.nfreqs,
                    param_names=np.array(self.param_names), **extra, **self.net.state())

    def load_state(self, state):
        self.mu = np.asarray(state["mu"], dtype=np.float64)
        self.sd = np.asarray(state["sd"], dtype=np.float64)
        self.residual_scatter = (np.asarray(state["residual_scatter"], dtype=np.float64)
                                 if "residual_scatter" in state else None)
        self.net.load_params(state["params"])


class _GraphedForward:
    def __init__(self, emu, batch, fused):
        t = D.torch()
        self.emu = emu
        self.batch = int(batch)
        dev = emu.net.device
        self.h_in = t.zeros((self.batch, INPUT_PAD), dtype=t.bfloat16).pin_memory()
        self.h_in_bits = self.h_in.view(t.int16).numpy()       # zero-copy view of the pinned inputs
        self.d_in = t.zeros((self.batch, INPUT_PAD), dtype=t.bfloat16, device=dev)
        self.h_out = t.zeros((emu.net.members, self.batch, emu.n_pad), dtype=t.float32).pin_memory()
        self.h_out_np = self.h_out.numpy()
        # the kernels' status word travels back with the outputs; it is cleared at the start of each
        # replay, so every call reports only its own kernels
        self.h_status = t.zeros(1, dtype=t.int32).pin_memory()
        self.h_status_np = self.h_status.numpy()
        self.stream = t.cuda.Stream(device=dev)
        self.fused = bool(fused)
        if self.fused and self.batch > N.MLP_FUSED_MAX_BATCH:
            raise ValueError(f"the fused forward takes at most {N.MLP_FUSED_MAX_BATCH} rows")
        with t.cuda.stream(self.stream):
            if self.fused:
                # one kernel node: it reads the pinned inputs and writes the pinned outputs and status
                # word itself (device-accessible host memory), so the graph has no copy nodes
                net = emu.net

                def launch():
                    N.call("hgb_mlp_forward_fused", ctypes.byref(net.struct), N.ptr(self.h_in), 0, self.batch,
                           N.ptr(self.h_out), N.ptr(self.h_status), N.stream_handle())

                launch()   # eager pass: the kernel's shared-memory attribute is set outside the capture
                self.stream.synchronize()
                net.check_status(int(self.h_status_np[0]))
                self.graph = t.cuda.CUDAGraph()
                with t.cuda.graph(self.graph, stream=self.stream):
                    launch()
            else:
                emu.net.forward(self.d_in, owner=self)   # eager pass: kernel attributes, this graph's buffers
                self.stream.synchronize()
                emu.net.check_status()
                self.graph = t.cuda.CUDAGraph()
                with t.cuda.graph(self.graph, stream=self.stream):
                    emu.net.status.t.zero_()
                    self.d_in.copy_(self.h_in, non_blocking=True)
                    out = emu.net.forward(self.d_in, owner=self)
                    self.h_out.copy_(out, non_blocking=True)
                    self.h_status.copy_(emu.net.status.t, non_blocking=True)
        self.stream.synchronize()

    def __call__(self, params):
        t = D.torch()
        u = self.emu.unit(params)
        q, npar = u.shape
        if q > self.batch:
            raise ValueError(f"at most {self.batch} queries per call")
        self.h_in_bits[:q, :npar] = bf16_bits(2.0 * u - 1.0).view(np.int16)
        if self.fused:
            self.h_status_np[0] = 0   # the kernel only sets bits
        cur = t.cuda.current_stream(self.emu.net.device)
        self.graph.replay()           # on the caller's current stream (a graph replays on any stream)
        cur.synchronize()
        self.emu.net.check_status(int(self.h_status_np[0]))
        out = self.h_out_np[:, :q, :self.emu.n_out].mean(axis=0, dtype=np.float64) * self.emu.sd + self.emu.mu
        return out.reshape(q, self.emu.nfreqs, 4)


class _NativeQuery:
    def __init__(self, emu, batch):
        t = D.torch()
        if not 1 <= int(batch) <= N.MLP_FUSED_MAX_BATCH:
            raise ValueError(f"batch must be in [1, {N.MLP_FUSED_MAX_BATCH}]")
        self.emu, self.batch = emu, int(batch)
        net = emu.net
        self.h_x = t.zeros((self.batch, net.dims[0]), dtype=t.int16).pin_memory()
        self.h_out = t.zeros((net.members, self.batch, net.dims[-1]), dtype=t.float32).pin_memory()
        self.h_status = t.zeros(1, dtype=t.int32).pin_memory()
        self.lo = np.ascontiguousarray(emu.lo, dtype=np.float64)
        self.hi = np.ascontiguousarray(emu.hi, dtype=np.float64)
        self.mu = np.ascontiguousarray(emu.mu, dtype=np.float64)
        self.sd = np.ascontiguousarray(emu.sd, dtype=np.float64)
        self.result = np.zeros((self.batch, emu.n_out), dtype=np.float64)
        self.fn = N.load().hgb_emulator_query
        self.args = [ctypes.byref(net.struct), None, 0, len(self.lo)] + [
            v.ctypes.data_as(ctypes.c_void_p) for v in (self.lo, self.hi, self.mu, self.sd)] + [
            emu.n_out, N.ptr(self.h_x), N.ptr(self.h_out), N.ptr(self.h_status),
            self.result.ctypes.data_as(ctypes.c_void_p)]

    def __call__(self, params):
        p = np.ascontiguousarray(np.atleast_2d(params), dtype=np.float64)
        nq = p.shape[0]
        if nq > self.batch or p.shape[1] != len(self.lo):
            raise ValueError(f"at most {self.batch} rows of {len(self.lo)} parameters")
        args = list(self.args)
        args[1] = p.ctypes.data_as(ctypes.c_void_p)
        args[2] = nq
        N.check(self.fn(*args, N.stream_handle()), "hgb_emulator_query")
        return self.result[:nq].reshape(nq, self.emu.nfreqs, 4).copy()


def sample_statistics(res):
    """``reduce`` hook of :func:`run_library`: the (F, 4) statistics of one sample's run_model dict."""
    return strain_statistics(res["hc_ss"], res["hc_bg"])


def library_statistics(results):
    """(S, F, 4) statistics of :func:`run_library` results, either run_model dicts or statistics
    already reduced by :func:`sample_statistics` (NaN rows for failed samples)."""
    rows = [None if r is None else (sample_statistics(r) if isinstance(r, dict) else np.asarray(r))
            for r in results]
    shape = next(r.shape for r in rows if r is not None)
    return np.stack([np.full(shape, np.nan) if r is None else r for r in rows])


def training_library(space, sam_shape=(91, 81, 101), nreals=500, nfreqs=40, seed=0, stats=None, **kwargs):
    """(S, F, 4) statistics of every sample of ``space``, from a batched GPU library run that keeps
    only the statistics of each sample (loudest source only; Philox keys from ``seed``)."""
    from .librarian import batch
    res = batch.run_library(space, shapes=sam_shape, nreals=nreals, nfreqs=nfreqs, nloudest=1, seed=seed,
                            reduce=sample_statistics, stats=stats, **kwargs)
    return library_statistics(res)


def boundary_space(space_cls, nsamples, seed=0):
    """A parameter space of ``nsamples`` points on the faces of ``space_cls``'s box: a Latin-hypercube
    draw (``seed``) with one coordinate per point, chosen uniformly, moved to its lower or upper
    bound.  A Latin hypercube rarely comes near the faces, so without such points the ensemble
    extrapolates there and its members disagree; added to a training library they put the faces
    inside the data.  (Two of the classic space's faces are physical limits, scatter = 0 and the
    shortest hardening time, so the box itself cannot be widened.)"""
    sp = space_cls(nsamples=nsamples, seed=seed)
    rng = np.random.default_rng([int(seed), 1])
    u = np.array(sp._uniform_samples, dtype=np.float64)
    k = rng.integers(0, u.shape[1], size=nsamples)
    u[np.arange(nsamples), k] = rng.integers(0, 2, size=nsamples).astype(np.float64)
    sp._uniform_samples = u
    sp.param_samples = np.stack([dist(u[:, ii]) for ii, dist in enumerate(sp._parameters)], axis=1)
    return sp


def sam_fallback(space, sam_shape=(91, 81, 101), nreals=500, nfreqs=40, nloudest=1, seed=0, precision="fp64"):
    """fallback(param_row) -> (F, 4): the plain GPU SAM at those parameters (grid arithmetic in
    ``precision``, see :meth:`Semi_Analytic_Model.gwb`)."""
    from .librarian import lib_tools

    def solve(row):
        params = dict(zip(space.param_names, np.asarray(row, dtype=np.float64)))
        sam, hard = space.model_for_params(params, sam_shape)
        res = lib_tools.run_model(sam, hard, nfreqs=nfreqs, nreals=nreals, nloudest=nloudest, gwb_flag=False,
                                  singles_flag=True, seed=seed, precision=precision)
        return strain_statistics(res["hc_ss"], res["hc_bg"])

    return solve


def timed(fn, *args, repeat=5):
    """Median wall time (s) of fn(*args) after one untimed call, with the device synchronised."""
    t = D.torch()
    fn(*args)
    t.cuda.synchronize()
    out = []
    for _ in range(repeat):
        t0 = time.perf_counter()
        fn(*args)
        t.cuda.synchronize()
        out.append(time.perf_counter() - t0)
    return float(np.median(out))
