"""Learned initial guess of the multigrid solve (binding of pgb_net_* in
libpamr_gb300): a 6-level convolutional encoder-decoder from the source rho
to a guess of u, trained on (rho, u) pairs the plain multigrid generates.
The kernels (BF16 tensor-core convolutions, training step) are in
pamr_amrd_gb300/csrc/pgb_net.cu; this module only sequences calls."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .solver import _check, lib

_vp, _dp = C.c_void_p, C.POINTER(C.c_double)
_bound = False


def _bind():
    global _bound
    L = lib()
    if _bound:
        return L
    L.pgb_net_create.argtypes = [C.c_int, C.c_ulonglong, C.POINTER(_vp)]
    L.pgb_net_destroy.argtypes = [_vp]
    L.pgb_net_destroy.restype = None
    L.pgb_net_set_scales.argtypes = [_vp, C.c_double, C.c_double]
    L.pgb_net_set_bias_free.argtypes = [_vp, C.c_int]
    L.pgb_net_num_params.argtypes = [_vp]
    L.pgb_net_num_params.restype = C.c_long
    L.pgb_net_params.argtypes = [_vp, C.c_int, C.POINTER(C.c_float), C.c_int]
    L.pgb_net_predict.argtypes = [_vp, _vp, _vp, _vp]
    L.pgb_net_predict_charge.argtypes = [_vp, _vp, _vp, _vp, C.c_double, _vp]
    L.pgb_net_rescale.argtypes = [_vp, _vp, _vp, C.c_double, _vp]
    L.pgb_net_rejected_guesses.argtypes = [_vp, C.POINTER(C.c_long)]
    L.pgb_net_loss_grad.argtypes = [_vp, _vp, _vp, _dp, _vp]
    L.pgb_net_train_step.argtypes = [_vp, _vp, _vp, C.c_float, _dp, _vp]
    L.pgb_conv3d_geometry.argtypes = [C.c_int] * 3 + [_vp, _vp]
    L.pgb_conv3d_pack_weights.argtypes = [_vp, _vp, C.c_int, C.c_int, C.c_int, _vp]
    L.pgb_conv3d_bf16.argtypes = [_vp] * 4 + [C.c_int] * 6 + [_vp, _vp]
    L.pgb_net_set_grid_cap.argtypes = [C.c_int]
    _bound = True
    return L


def set_grid_cap(ctas: int):
    """at most `ctas` CTAs for the persistent tensor-core convolution (0: a
    full wave): a prediction that runs beside a solve leaves it the other
    SMs; the results do not depend on it"""
    _check(_bind().pgb_net_set_grid_cap(ctas))


def conv_lib():
    """the library with the tensor-core convolution entry points bound"""
    return _bind()


class Net:
    """n: grid points per side of the solve (n-1 a multiple of 32, 65 <= n <= 513)"""

    # levels and channels per level (pgb_net.cu: NLEV, LCH)
    NLEV = 6
    LCH = (16, 32, 64, 64, 64, 64)

    @classmethod
    def dec_layer(cls, v: int) -> int:
        """index of the tensor-core layer of level v's decoder"""
        return 2 * (cls.NLEV - 1) + 1 + (cls.NLEV - 2 - v)

    @classmethod
    def layers(cls):
        """layer table in parameter order: (name, cin, cout)"""
        ch = cls.LCH
        tcl = [(ch[0], ch[0])]
        for v in range(1, cls.NLEV):
            tcl += [(ch[v - 1], ch[v]), (ch[v], ch[v])]
        tcl += [(ch[v], ch[max(v - 1, 0)]) for v in range(cls.NLEV - 2, -1, -1)]
        return [("in", 1, ch[0])] + [(f"tc{i}", a, b) for i, (a, b) in enumerate(tcl)] + [("out", ch[0], 1)]

    def __init__(self, n: int, seed: int = 1):
        L = _bind()
        h = _vp()
        _check(L.pgb_net_create(n, seed, C.byref(h)))
        self.h, self.n = h, n
        self.s_in = self.s_out = 1.0
        if self.num_params() != sum(27 * ci * co + co for _, ci, co in self.LAYERS):
            raise RuntimeError("pgb_net: layer table of the library and of learned.py differ")

    def close(self):
        if self.h:
            lib().pgb_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_scales(self, s_in: float, s_out: float):
        self.s_in, self.s_out = s_in, s_out
        _check(lib().pgb_net_set_scales(self.h, s_in, s_out))

    def set_bias_free(self, on: bool = True):
        _check(lib().pgb_net_set_bias_free(self.h, 1 if on else 0))

    def num_params(self) -> int:
        return int(lib().pgb_net_num_params(self.h))

    def params(self, which: int = 0) -> np.ndarray:
        out = np.zeros(self.num_params(), dtype=np.float32)
        _check(lib().pgb_net_params(self.h, which, out.ctypes.data_as(C.POINTER(C.c_float)), 0))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(lib().pgb_net_params(self.h, 0, p.ctypes.data_as(C.POINTER(C.c_float)), 1))

    def split(self, flat: np.ndarray) -> dict:
        """parameter vector -> {name: (w[27][cin][cout], b[cout])}"""
        out, o = {}, 0
        for name, ci, co in self.LAYERS:
            w = flat[o:o + 27 * ci * co].reshape(27, ci, co)
            o += 27 * ci * co
            out[name] = (w, flat[o:o + co])
            o += co
        return out

    def predict(self, rho_ptr: int, u_ptr: int, stream=None):
        _check(lib().pgb_net_predict(self.h, rho_ptr, u_ptr, stream))

    def predict_charge(self, rho_ptr: int, u_ptr: int, q_ptr: int, gain: float, stream=None):
        """predict with s_in = 1/q, s_out = gain q read from the device value
        at q_ptr (computed on the same stream)"""
        _check(lib().pgb_net_predict_charge(self.h, rho_ptr, u_ptr, q_ptr, gain, stream))

    def rescale(self, rho_ptr: int, u_ptr: int, h: float, stream=None):
        """energy-norm optimal amplitude of the guess (pgb_net_rescale); a
        guess that is not finite or needs an absurd amplitude becomes u = 0"""
        _check(lib().pgb_net_rescale(self.h, rho_ptr, u_ptr, h, stream))

    def rejected_guesses(self) -> int:
        n = C.c_long()
        _check(lib().pgb_net_rejected_guesses(self.h, C.byref(n)))
        return n.value

    def loss_grad(self, rho_ptr: int, ut_ptr: int, stream=None) -> float:
        loss = C.c_double()
        _check(lib().pgb_net_loss_grad(self.h, rho_ptr, ut_ptr, C.byref(loss), stream))
        return loss.value

    def train_step(self, rho_ptr: int, ut_ptr: int, lr: float, stream=None, want_loss: bool = True):
        loss = C.c_double()
        _check(lib().pgb_net_train_step(self.h, rho_ptr, ut_ptr, lr, C.byref(loss) if want_loss else None,
                                        stream))
        return loss.value if want_loss else None


Net.LAYERS = Net.layers()


# ------------------------------------------------ data, training, use ----
def rho_on_device(n: int, blobs, torch):
    """poisson3d's source on the device (FP64, x fastest), from its blobs"""
    x = torch.linspace(-10.0, 10.0, n, dtype=torch.float64, device="cuda")
    Z, Y, X = torch.meshgrid(x, x, x, indexing="ij")
    r = torch.zeros_like(X)
    for a, w, c in blobs:
        r += a * torch.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / (w * w))
    return r.reshape(-1).contiguous()


def source_charge(rho, h: float) -> float:
    """sum |rho| h^3: the scale of a sample (rho a device tensor)"""
    return max(float(rho.abs().sum()) * h ** 3, 1e-300)


class Scaled:
    """The equation is linear in rho: the net is made bias-free (positively
    homogeneous, so scaling rho scales its guess exactly) and every sample
    is scaled by its own source charge Q: the net reads rho / Q and
    predicts u / (gain * Q), `gain` (max |u| / Q over the training pairs)
    fixed at training, so that inputs and targets are of order one
    whatever the source's size."""

    def __init__(self, net: Net, gain: float, h: float):
        self.net, self.gain, self.h = net, gain, h
        net.set_bias_free(True)

    def _scale(self, rho) -> None:
        q = source_charge(rho, self.h)
        self.net.set_scales(1.0 / q, self.gain * q)

    def train_step(self, rho, ut, lr: float, want_loss: bool = True):
        self._scale(rho)
        return self.net.train_step(rho.data_ptr(), ut.data_ptr(), lr, want_loss=want_loss)

    def predict(self, rho, u, stream=None, rescale: bool = True):
        """the guess of u for source rho (device tensors), its amplitude set
        by the energy norm unless rescale is False. The charge that scales
        rho and the guess is summed on the device, on the prediction's
        stream, so the host does not wait for it."""
        import torch
        ts = torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()
        with torch.cuda.stream(ts):
            self._q = rho.abs().sum() * (self.h ** 3)   # kept until the next prediction
            self.net.predict_charge(rho.data_ptr(), u.data_ptr(), self._q.data_ptr(), self.gain,
                                    ts.cuda_stream)
            if rescale:
                self.net.rescale(rho.data_ptr(), u.data_ptr(), self.h, ts.cuda_stream)


def make_dataset(n: int, seeds, torch, cycles: int = 12, precision: int = 1):
    """(rho, u) training pairs from the plain multigrid: for each seed the
    poisson3d source and the solution after `cycles` V-cycles (about 1e-12
    of the initial residual); u kept as FP32 on the device"""
    import copy
    from . import workloads as W
    from .solver import Solver
    case = copy.deepcopy(W.poisson3d(n, seed=0, rel_tol=0))
    case.params.precision = precision
    case.params.tol = 0.0
    case.params.max_iter = cycles
    case.params.min_iter = cycles
    s = Solver(case)
    zero = torch.zeros(n ** 3, dtype=torch.float64, device="cuda")
    u = torch.empty(n ** 3, dtype=torch.float64, device="cuda")
    blobs, U = [], torch.empty(len(seeds), n ** 3, dtype=torch.float32, device="cuda")
    st = torch.cuda.ExternalStream(s.stream())
    torch.cuda.synchronize()
    for k, seed in enumerate(seeds):
        b = W.poisson3d_blobs(seed)
        with torch.cuda.stream(st):   # ordered before the solver's copy of it
            rho = rho_on_device(n, b, torch)
        s.set_inputs_device([zero.data_ptr()], [rho.data_ptr()])
        s.solve()
        _check(lib().pgb_get_grid_device(s.h, 0, u.data_ptr()))
        torch.cuda.synchronize()
        U[k] = u.float()
        blobs.append(b)
    s.close()
    return blobs, U


def moving_blobs(seed: int, step: int, dt: float = 0.05):
    """the poisson3d source of `seed` with its Gaussians drifting: centre
    c + v t at t = step dt, with seeded velocities v in U(-1, 1)^3 (units of
    the domain [-10, 10]^3 per unit time) -- the source a time-stepped run
    hands its elliptic solve at each coarse step"""
    from . import workloads as W
    rng = W.SplitMix64(0x5EED0009 + seed)
    out = []
    for (a, w, c) in W.poisson3d_blobs(seed):
        v = (rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-1, 1))
        t = step * dt
        out.append((a, w, tuple(c[d] + v[d] * t for d in range(3))))
    return out


def make_sequence_dataset(n: int, runs, steps: int, torch, cycles: int = 12, precision: int = 1):
    """(rho, u) training pairs the plain multigrid produces along
    time-stepped runs, as the elliptic solves of a Berger-Oliger evolution
    (amrd/evolve.c:279-288) would: for each run (seed) and coarse step, the
    drifting source of moving_blobs is solved by `cycles` V-cycles started
    from the previous step's solution (AMRD starts each solve from the last
    one), and the pair is kept; u as FP32 on the device"""
    import copy
    from . import workloads as W
    from .solver import Solver
    case = copy.deepcopy(W.poisson3d(n, seed=0, rel_tol=0))
    case.params.precision = precision
    case.params.tol = 0.0
    case.params.max_iter = cycles
    case.params.min_iter = cycles
    s = Solver(case)
    runs = list(runs)
    u = torch.zeros(n ** 3, dtype=torch.float64, device="cuda")
    blobs, U = [], torch.empty(len(runs) * steps, n ** 3, dtype=torch.float32, device="cuda")
    st = torch.cuda.ExternalStream(s.stream())
    torch.cuda.synchronize()
    k = 0
    for seed in runs:
        u.zero_()
        for step in range(steps):
            b = moving_blobs(seed, step)
            with torch.cuda.stream(st):   # ordered before the solver's copy of it
                rho = rho_on_device(n, b, torch)
            s.set_inputs_device([u.data_ptr()], [rho.data_ptr()])
            s.solve()
            _check(lib().pgb_get_grid_device(s.h, 0, u.data_ptr()))
            torch.cuda.synchronize()
            U[k] = u.float()
            blobs.append(b)
            k += 1
    s.close()
    return blobs, U


def fit_gain(n: int, blobs, U, torch) -> float:
    h = 20.0 / (n - 1)
    return max(float(U[i].abs().max()) / source_charge(rho_on_device(n, b, torch), h) for i, b in enumerate(blobs))


def train(model: Scaled, blobs, U, torch, epochs: int = 2, lr: float = 1e-3, lr_end: float = 1e-5, seed: int = 0,
          log=None):
    """Adam over the pairs, one pair per step, cosine learning-rate decay;
    returns the mean loss of each epoch"""
    n, N = model.net.n, len(blobs)
    order = np.random.default_rng(seed)
    steps, k, out = epochs * N, 0, []
    for ep in range(epochs):
        tot = 0.0
        for i in order.permutation(N):
            rate = lr_end + 0.5 * (lr - lr_end) * (1 + np.cos(np.pi * k / max(1, steps - 1)))
            tot += model.train_step(rho_on_device(n, blobs[i], torch), U[i], float(rate))
            k += 1
        out.append(tot / N)
        if log:
            log(f"epoch {ep}: mean loss {out[-1]:.4e}")
    return out


class GuessPolicy:
    """Uses the net's guess as the initial u of a solve while it pays. The
    plain solve always runs to tolerance after the guess, so a bad guess
    costs time, never accuracy. A guessed solve that needs no fewer
    V-cycles than the last unguessed one, or takes no less time (the
    prediction included), is a strike; `patience` strikes in a row send
    the policy back to the plain initial guess (u = 0) for good."""

    def __init__(self, patience: int = 2):
        self.patience, self.strikes, self.enabled = patience, 0, True
        self.plain_cycles = self.plain_ms = None

    def use_guess(self) -> bool:
        return self.enabled and self.plain_cycles is not None

    def record(self, cycles: int, guessed: bool, ms: float | None = None):
        if not guessed:
            self.plain_cycles, self.plain_ms = cycles, ms
            return
        slower = ms is not None and self.plain_ms is not None and ms >= self.plain_ms
        if self.plain_cycles is not None and (cycles >= self.plain_cycles or slower):
            self.strikes += 1
            if self.strikes >= self.patience:
                self.enabled = False
        else:
            self.strikes = 0
