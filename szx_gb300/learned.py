"""Learned fixed-rate selection and batched fields on the GPU (torch tensors).

* ``Batch``: a compress plan over many device float32 fields
  (SZxG_batch_create / run / set_bounds), its feature rows
  (SZxG_batch_features) and the fixed-rate driver (SZxG_batch_fixed_rate).
* ``Mlp``: the bound-predicting network (SZxG_mlp_*), trained on the GPU by
  the library's own forward / backward / Adam kernels.
* ``synthetic_fields`` / ``training_set`` / ``train``: the training corpus:
  seeded fields, and (features, bound, ratio) triples measured by real
  compress passes of the codec (the label: the measured ratio's miss of the
  target at the bound the sampled model picks).

The reference's fixed-rate mode searches an analytic model of every 10th
block (szx/src/szx_float.cc:684-832, 921-949); here the decision is judged by
compressing the field for real.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import StreamInfo, lib

FEATURES = 32


class SZxError(RuntimeError):
    pass


def _check(rc: int, what: str):
    if rc:
        raise SZxError(f"{what}: {lib().SZxG_error_string(rc).decode()} ({rc})")


class _Field(C.Structure):
    """SZxG_Field."""
    _fields_ = [("in_", C.c_void_p), ("nbEle", C.c_size_t), ("inBytes", C.c_size_t), ("absErrBound", C.c_float),
                ("reserved", C.c_int), ("out", C.c_void_p), ("outCapacity", C.c_size_t)]


def _stream_of(t):
    import torch
    return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


class Batch:
    """Compress plan over device float32 fields (fastMode 2 by default, the
    layout of the reference's fixed-rate streams; blockSize 128)."""

    def __init__(self, fields, bounds=None, fastMode: int = 2, blockSize: int = 128):
        import torch
        self.torch = torch
        self.fields = [f.contiguous() for f in fields]
        for f in self.fields:
            if f.dtype != torch.float32 or not f.is_cuda:
                raise ValueError("fields must be float32 CUDA tensors")
        self.mode, self.bs, self.nf = fastMode, blockSize, len(self.fields)
        self.n = np.array([f.numel() for f in self.fields], dtype=np.int64)
        L = lib()
        self.outs = []
        tab = (_Field * self.nf)()
        for k, f in enumerate(self.fields):
            cap = L.SZxG_compress_bound(fastMode, 0, f.numel(), blockSize)
            o = torch.empty(cap, dtype=torch.uint8, device=f.device)
            self.outs.append(o)
            eb = float(bounds[k]) if bounds is not None else 1.0
            tab[k] = _Field(f.data_ptr(), f.numel(), 0, eb, 0, o.data_ptr(), cap)
        self.h = L.SZxG_batch_create(0, fastMode, 0, blockSize, self.nf, C.cast(tab, C.c_void_p))
        if not self.h:
            _check(L.SZxG_get_last_error(), "SZxG_batch_create")
        self.info = torch.zeros(self.nf * C.sizeof(StreamInfo), dtype=torch.uint8, device=self.fields[0].device)

    def close(self):
        if self.h:
            lib().SZxG_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _s(self):
        return _stream_of(self.fields[0])

    def set_bounds(self, bounds, idx=None):
        eb = np.ascontiguousarray(bounds, dtype=np.float32)
        if idx is None:
            _check(lib().SZxG_batch_set_bounds(self.h, self.nf, None, eb.ctypes.data_as(C.POINTER(C.c_float)),
                                               self._s()), "SZxG_batch_set_bounds")
        else:
            ix = np.ascontiguousarray(idx, dtype=np.int32)
            _check(lib().SZxG_batch_set_bounds(self.h, len(ix), ix.ctypes.data_as(C.POINTER(C.c_int)),
                                               eb.ctypes.data_as(C.POINTER(C.c_float)), self._s()),
                   "SZxG_batch_set_bounds")

    def run(self):
        _check(lib().SZxG_batch_run(self.h, C.c_void_p(self.info.data_ptr()), self._s()), "SZxG_batch_run")

    def infos(self):
        self.torch.cuda.synchronize()
        raw = self.info.cpu().numpy().tobytes()
        k = C.sizeof(StreamInfo)
        return [StreamInfo.from_buffer_copy(raw[i * k:(i + 1) * k]) for i in range(self.nf)]

    def sizes(self) -> np.ndarray:
        return np.array([i.size for i in self.infos()], dtype=np.int64)

    def stream(self, k: int) -> bytes:
        i = self.infos()[k]
        return self.outs[k][i.offset:i.offset + i.size].cpu().numpy().tobytes()

    def features(self, rows, targets):
        """(X [len(rows), 32] device tensor, sampled range per field)."""
        torch = self.torch
        r = np.ascontiguousarray(rows, dtype=np.int32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        X = torch.empty((len(r), FEATURES), dtype=torch.float32, device=self.fields[0].device)
        rng = np.zeros(self.nf, dtype=np.float32)
        _check(lib().SZxG_batch_features(self.h, len(r), r.ctypes.data_as(C.POINTER(C.c_int)),
                                         t.ctypes.data_as(C.POINTER(C.c_float)), C.c_void_p(X.data_ptr()),
                                         rng.ctypes.data_as(C.POINTER(C.c_float)), self._s()),
               "SZxG_batch_features")
        return X, rng

    def fixed_rate(self, targets, mlp: "Mlp | None" = None, tolerance: float = 0.05, max_passes: int = 20):
        """Bounds for every field's target ratio (NULL model: bisection).
        Returns (bounds, achieved ratios, passes) and leaves the streams in
        the plan's output buffers."""
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(targets, np.float32), (self.nf,)))
        eb = np.zeros(self.nf, np.float32)
        cr = np.zeros(self.nf, np.float32)
        ps = np.zeros(self.nf, np.int32)
        fp = C.POINTER(C.c_float)
        _check(lib().SZxG_batch_fixed_rate(self.h, mlp.h if mlp is not None else None, t.ctypes.data_as(fp),
                                           tolerance, max_passes, eb.ctypes.data_as(fp), cr.ctypes.data_as(fp),
                                           ps.ctypes.data_as(C.POINTER(C.c_int)), C.c_void_p(self.info.data_ptr()),
                                           self._s()), "SZxG_batch_fixed_rate")
        return eb, cr, ps


class Mlp:
    """The 32-64-64-64-1 GELU bound predictor (parameters on the device)."""

    def __init__(self, seed: int = 0, params: np.ndarray | None = None):
        L = lib()
        self.count = int(L.SZxG_mlp_param_count())
        self.h = L.SZxG_mlp_create(seed)
        if not self.h:
            _check(L.SZxG_get_last_error(), "SZxG_mlp_create")
        if params is not None:
            self.set_params(params)

    def close(self):
        if self.h:
            lib().SZxG_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        p = np.zeros(self.count, np.float32)
        _check(lib().SZxG_mlp_get_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float)), p.size), "get_params")
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(lib().SZxG_mlp_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float)), p.size), "set_params")

    def forward(self, X):
        import torch
        X = X.contiguous()
        out = torch.empty(X.shape[0], dtype=torch.float32, device=X.device)
        _check(lib().SZxG_mlp_forward(self.h, C.c_void_p(X.data_ptr()), X.shape[0], C.c_void_p(out.data_ptr()),
                                      _stream_of(X)), "SZxG_mlp_forward")
        return out

    def gradient(self, X, y):
        """(mean squared error, gradient of the trainable parameters)."""
        import torch
        X, y = X.contiguous(), y.contiguous()
        g = torch.empty(self.count - 64, dtype=torch.float32, device=X.device)
        loss = C.c_float()
        _check(lib().SZxG_mlp_gradient(self.h, C.c_void_p(X.data_ptr()), C.c_void_p(y.data_ptr()), X.shape[0],
                                       C.c_void_p(g.data_ptr()), C.byref(loss), _stream_of(X)), "SZxG_mlp_gradient")
        return loss.value, g

    def train(self, X, y, epochs: int = 200, batch: int = 512, lr: float = 2e-3, seed: int = 0) -> float:
        X, y = X.contiguous(), y.contiguous()
        loss = C.c_float()
        _check(lib().SZxG_mlp_train(self.h, C.c_void_p(X.data_ptr()), C.c_void_p(y.data_ptr()), X.shape[0], epochs,
                                    batch, lr, seed, C.byref(loss), _stream_of(X)), "SZxG_mlp_train")
        return loss.value


# ------------------------------------------------------------------ training corpus

def synthetic_fields(nf: int, lo_exp: float, hi_exp: float, seed: int, device="cuda"):
    """nf seeded float32 fields on the device, sizes log-uniform in
    [2^lo_exp, 2^hi_exp]: 1-D k^-5/3 spectral fields, piecewise-constant
    levels (runs of 64..4096) with noise at 1e-3 of the level spread, and white
    noise, each scaled by 10^U(-2,2) and offset.  Returns (fields, kinds)."""
    import torch
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(2.0 ** lo_exp), np.log(2.0 ** hi_exp), nf)).astype(np.int64)
    kinds = rng.integers(0, 3, nf)
    scales = 10.0 ** rng.uniform(-2, 2, nf)
    offs = rng.uniform(-3, 3, nf)
    g = torch.Generator(device=device).manual_seed(int(seed))
    out = []
    for n, kind, sc, of in zip(sizes, kinds, scales, offs):
        n = int(n)
        if kind == 0:
            n2 = 1 << (n - 1).bit_length()
            nh = n2 // 2 + 1
            k = torch.arange(nh, device=device, dtype=torch.float32)
            k[0] = 1.0
            amp = k ** (-5.0 / 6.0)
            amp[0] = 0.0
            z = torch.complex(torch.randn(nh, generator=g, device=device),
                              torch.randn(nh, generator=g, device=device)) * amp
            x = torch.fft.irfft(z, n=n2)[:n]
            x = (x - x.mean()) / (x.std() + 1e-30)
        elif kind == 1:
            run = int(rng.integers(64, 4097))
            lv = torch.randn(n // run + 1, generator=g, device=device)
            x = torch.repeat_interleave(lv, run)[:n] + 1e-3 * torch.randn(n, generator=g, device=device)
        else:
            x = torch.randn(n, generator=g, device=device)
        out.append((x * float(sc) + float(of * sc)).float().contiguous())
    return out, kinds


def training_set(batch: Batch, passes: int = 40, seed: int = 0):
    """(X, miss, ratio) from real compress passes of the batch.  In each pass
    every field draws a target ratio log-uniform in [2, 64], is compressed at
    its sampled curve's crossing for that target (feature 1), and gives one
    row: its feature row for the target, labelled with the miss
    log2(measured ratio / target).  Rows whose target the codec cannot reach
    (|miss| > 1.5, a jump of the ratio over the target) are dropped."""
    torch = batch.torch
    rng = np.random.default_rng(seed)
    nf = batch.nf
    allf = np.arange(nf)
    Xs, ms, crs = [], [], []
    safe = None
    for p in range(passes):
        tg = np.exp2(rng.uniform(1.0, 6.0, nf)).astype(np.float32)
        Xp, rg = batch.features(allf, tg)
        if safe is None:
            safe = np.where(rg > 0, rg, 1.0).astype(np.float64)
        ys = Xp[:, 1].double().cpu().numpy()
        batch.set_bounds((safe * np.exp2(ys)).astype(np.float32))
        batch.run()
        cr = batch.n * 4.0 / batch.sizes()
        miss = np.log2(cr / tg.astype(np.float64))
        keep = np.abs(miss) <= 1.5
        Xs.append(Xp[torch.tensor(keep, device=Xp.device)])
        ms.append(miss[keep])
        crs.append(cr[keep])
    X = torch.cat(Xs)
    return X, torch.tensor(np.concatenate(ms).astype(np.float32), device=X.device), np.concatenate(crs)


def train(X, y, seed: int = 0, epochs: int = 300, batch: int = 512, lr: float = 2e-3):
    """A fresh network trained on (X, y); returns (model, final training loss)."""
    m = Mlp(seed)
    loss = m.train(X, y, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return m, loss
