"""ctypes binding of ``libqmc.so`` (the C ABI declared in ``include/qmc.h``).

The library is built in-tree by ``jaqmc_gb300.build``.  Loading fails loudly
when it is missing or when no sm_103 device is present: there is no CPU
fallback on the product path.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np
import torch

LIB_PATH = Path(__file__).resolve().parent / "libqmc.so"

QMC_OK = 0
STATUS = {0: "OK", 1: "ARG", 2: "SHAPE", 3: "NUMERIC", 4: "TIMEOUT", 5: "CUDA", 6: "WORKSPACE",
          7: "UNSUPPORTED"}
PRECISION = {"fp32": 0, "plain": 0, "mixed": 1, "bf16": 1}
ENVELOPE = {"isotropic": 0, "abs_isotropic": 1, "diagonal": 2, "null": 3}
OP_FORWARD, OP_LOCAL_ENERGY, OP_MH, OP_GRAD = 0, 1, 2, 3
FLAG_NONFINITE, FLAG_REFACTOR, FLAG_SINGULAR = 1, 2, 4
MAX_LAYERS = 8


class QmcError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"qmc status {STATUS.get(status, status)}: {msg}")
        self.status = status


class FermiNetConfigC(C.Structure):
    _fields_ = [("n_up", C.c_int), ("n_down", C.c_int), ("n_atoms", C.c_int), ("ndets", C.c_int),
                ("n_layers", C.c_int), ("hidden_single", C.c_int * MAX_LAYERS),
                ("hidden_double", C.c_int * MAX_LAYERS), ("envelope", C.c_int),
                ("orbitals_spin_split", C.c_int), ("precision", C.c_int)]


class PsiformerConfigC(C.Structure):
    _fields_ = [("n_up", C.c_int), ("n_down", C.c_int), ("n_atoms", C.c_int), ("ndets", C.c_int),
                ("n_layers", C.c_int), ("n_heads", C.c_int), ("head_dim", C.c_int), ("n_mlp", C.c_int),
                ("mlp_dims", C.c_int * 4), ("envelope", C.c_int), ("orbitals_spin_split", C.c_int),
                ("jastrow", C.c_int), ("precision", C.c_int)]


class LapNetConfigC(C.Structure):
    _fields_ = [("n_up", C.c_int), ("n_down", C.c_int), ("n_atoms", C.c_int), ("ndets", C.c_int),
                ("n_layers", C.c_int), ("n_heads", C.c_int), ("head_dim", C.c_int),
                ("num_local_updates", C.c_int), ("use_input_bias", C.c_int), ("use_backbone_bias", C.c_int),
                ("envelope", C.c_int), ("orbitals_spin_split", C.c_int), ("jastrow", C.c_int),
                ("precision", C.c_int)]


class LayerTapC(C.Structure):
    _fields_ = [("kind", C.c_int), ("rows_per_walker", C.c_int), ("in_cols", C.c_int), ("out_cols", C.c_int),
                ("has_bias", C.c_int), ("kernel_offset", C.c_size_t), ("bias_offset", C.c_size_t),
                ("in_offset", C.c_size_t), ("out_offset", C.c_size_t)]


TAP_DENSE, TAP_DIAGONAL = 0, 1

_lib = None
_lock = threading.Lock()

# name -> (restype, argtypes)
_SIGS = {
    "qmc_last_error": (C.c_char_p, []),
    "qmc_device_check": (C.c_int, [C.POINTER(C.c_int)] * 3),
    "qmc_ferminet_create": (C.c_int, [C.POINTER(FermiNetConfigC), C.c_void_p, C.c_void_p,
                                      C.POINTER(C.c_void_p)]),
    "qmc_psiformer_create": (C.c_int, [C.POINTER(PsiformerConfigC), C.c_void_p, C.c_void_p,
                                       C.POINTER(C.c_void_p)]),
    "qmc_lapnet_create": (C.c_int, [C.POINTER(LapNetConfigC), C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "qmc_model_destroy": (C.c_int, [C.c_void_p]),
    "qmc_param_count": (C.c_size_t, [C.c_void_p]),
    "qmc_model_set_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "qmc_model_set_precision": (C.c_int, [C.c_void_p, C.c_int]),
    "qmc_model_set_det_guard": (C.c_int, [C.c_void_p, C.c_int]),
    "qmc_workspace_size": (C.c_size_t, [C.c_void_p, C.c_int, C.c_int]),
    "qmc_forward": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_void_p, C.c_size_t, C.c_void_p]),
    "qmc_forward_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p]),
    "qmc_local_energy": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                   C.c_void_p]),
    "qmc_mh_steps": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_uint64, C.c_uint64,
                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "qmc_mh_steps_resident": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_uint64, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_size_t, C.c_void_p]),
    "qmc_tangent_rows": (C.c_int, [C.c_void_p, C.c_int]),
    "qmc_mh_draws": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_uint64, C.c_uint64, C.c_void_p,
                               C.c_void_p, C.c_void_p]),
    "qmc_reduce_mean_var": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "qmc_grad": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                           C.c_void_p, C.c_size_t, C.c_void_p]),
    "qmc_model_set_grad_budget": (C.c_int, [C.c_void_p, C.c_size_t]),
    "qmc_layer_taps": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(LayerTapC), C.c_int, C.POINTER(C.c_size_t)]),
    "qmc_grad_taps": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p,
                                C.c_size_t, C.c_void_p]),
    "qmc_model_set_energy_budget": (C.c_int, [C.c_void_p, C.c_size_t]),
    "qmc_model_check_error": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "qmc_profile_enable": (C.c_int, [C.c_int]),
    "qmc_profile_read": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p]),
    "qmc_ecp_workspace_size": (C.c_size_t, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]),
    "qmc_ecp_energy": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                 C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64, C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "qmc_ffma_throughput": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_double), C.c_void_p]),
    "qmc_mma_throughput": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_double), C.c_void_p]),
    "qmc_mh_steps_grouped": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                       C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_size_t, C.c_void_p]),
    "qmc_reduce_mean_var_segments": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
}


def exported_symbols():
    """Names the library must export (every entry point of include/qmc.h)."""
    return list(_SIGS)


def load(path: Path | None = None):
    """Load ``libqmc.so`` (no device needed) and bind the signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path or LIB_PATH)
        if not p.exists():
            raise FileNotFoundError(
                f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "or `python -m jaqmc_gb300.build` (there is no CPU fallback)")
        lib = C.CDLL(str(p))
        for name, (res, args) in _SIGS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib


def check(status: int):
    if status != QMC_OK:
        raise QmcError(status, load().qmc_last_error().decode())


def ptr(t) -> int | None:
    if t is None:
        return None
    if isinstance(t, torch.Tensor):
        if not t.is_cuda:
            raise ValueError("expected a CUDA tensor")
        if not t.is_contiguous():
            raise ValueError("expected a contiguous tensor")
        return t.data_ptr()
    return int(t)


def stream_handle(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def device_check():
    lib = load()
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    check(lib.qmc_device_check(C.byref(a), C.byref(b), C.byref(c)))
    return a.value, b.value, c.value


class Workspace:
    """Caller-owned scratch buffers, grown on demand (never inside a step)."""

    def __init__(self, device):
        self.device = device
        self.buf = None

    def get(self, nbytes: int) -> torch.Tensor:
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=self.device)
        return self.buf


class NativeFermiNet:
    """One ``qmc_model`` handle: a FermiNet for one molecule on one device."""

    def _open(self, device):
        self.lib = load()
        if not torch.cuda.is_available():
            raise RuntimeError("no CUDA device: the qmc library has no CPU fallback")
        dev = torch.device(device or "cuda")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        torch.cuda.set_device(self.device)
        device_check()

    def __init__(self, cfg, atoms, charges, precision="fp32", device=None):
        self._open(device)
        lib = self.lib
        c = FermiNetConfigC()
        c.n_up, c.n_down = int(cfg.nspins[0]), int(cfg.nspins[1])
        atoms = np.ascontiguousarray(np.asarray(atoms, np.float32).reshape(-1, 3))
        charges = np.ascontiguousarray(np.asarray(charges, np.float32).reshape(-1))
        c.n_atoms = atoms.shape[0]
        c.ndets = int(cfg.ndets)
        L = len(cfg.hidden_dims_single)
        c.n_layers = L
        for i in range(L):
            c.hidden_single[i] = int(cfg.hidden_dims_single[i])
            c.hidden_double[i] = int(cfg.hidden_dims_double[i])
        c.envelope = ENVELOPE[str(cfg.envelope)]
        c.orbitals_spin_split = int(bool(cfg.orbitals_spin_split))
        c.precision = PRECISION[precision]
        if getattr(cfg, "use_last_layer", False):
            raise QmcError(7, "use_last_layer=True is not supported")
        h = C.c_void_p()
        check(lib.qmc_ferminet_create(C.byref(c), atoms.ctypes.data, charges.ctypes.data, C.byref(h)))
        self._finish(h, c.n_up + c.n_down, precision)

    def _finish(self, h, n, precision):
        self.h = h
        self.n = n
        self.precision = precision
        self.ws = Workspace(self.device)

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            try:
                self.lib.qmc_model_destroy(h)
            except Exception:
                pass
            self.h = None

    @property
    def param_count(self) -> int:
        return int(self.lib.qmc_param_count(self.h))

    def set_det_guard(self, mode: int):
        """FP64 re-evaluation of cancelling determinants in the local energy:
        1 on, 0 off, -1 by precision (on for FP32, off for mixed)."""
        check(self.lib.qmc_model_set_det_guard(self.h, int(mode)))

    def set_precision(self, precision: str):
        check(self.lib.qmc_model_set_precision(self.h, PRECISION[precision]))
        self.precision = precision

    def set_params(self, flat: torch.Tensor, stream=None):
        flat = flat.to(device=self.device, dtype=torch.float32).contiguous()
        if flat.numel() != self.param_count:
            raise QmcError(2, f"expected {self.param_count} parameters, got {flat.numel()}")
        check(self.lib.qmc_model_set_params(self.h, ptr(flat), stream_handle(stream)))
        self._params = flat  # keep alive until the copy has run

    def check_error(self) -> int:
        """Device error word of the bounded waits (0 = none); raises on error."""
        code = C.c_int(0)
        check(self.lib.qmc_model_check_error(self.h, C.byref(code)))
        return code.value

    def workspace(self, op: int, batch: int):
        nb = int(self.lib.qmc_workspace_size(self.h, op, batch))
        return self.ws.get(nb), nb

    def _elec(self, electrons):
        e = electrons
        if e.dtype != torch.float32 or not e.is_cuda or not e.is_contiguous():
            raise ValueError("electrons must be a contiguous float32 CUDA tensor (B, n, 3)")
        if e.dim() != 3 or e.shape[1] != self.n or e.shape[2] != 3:
            raise ValueError(f"electrons must have shape (B, {self.n}, 3), got {tuple(e.shape)}")
        return e

    def forward(self, electrons, stream=None):
        e = self._elec(electrons)
        B = e.shape[0]
        lp = torch.empty(B, dtype=torch.float32, device=self.device)
        sg = torch.empty_like(lp)
        fl = torch.empty(B, dtype=torch.uint8, device=self.device)
        ws, nb = self.workspace(OP_FORWARD, B)
        check(self.lib.qmc_forward(self.h, B, ptr(e), ptr(lp), ptr(sg), ptr(fl), ptr(ws), ws.numel(),
                                   stream_handle(stream)))
        return lp, sg, fl

    def local_energy(self, electrons, stream=None):
        e = self._elec(electrons)
        B = e.shape[0]
        out = torch.empty((4, B), dtype=torch.float32, device=self.device)
        fl = torch.empty(B, dtype=torch.uint8, device=self.device)
        ws, nb = self.workspace(OP_LOCAL_ENERGY, B)
        check(self.lib.qmc_local_energy(self.h, B, ptr(e), ptr(out[0]), ptr(out[1]), ptr(out[2]),
                                        ptr(out[3]), ptr(fl), ptr(ws), ws.numel(), stream_handle(stream)))
        return {"e_local": out[0], "kinetic": out[1], "potential": out[2], "logpsi": out[3], "flags": fl}

    def mh_steps(self, electrons, steps, stddev, seed, counter, log_prob=None, accepts=None,
                 normals=None, uniforms=None, stream=None):
        e = self._elec(electrons)
        B = e.shape[0]
        if log_prob is None:
            log_prob = torch.empty(B, dtype=torch.float32, device=self.device)
        if accepts is None:
            accepts = torch.zeros(B, dtype=torch.int32, device=self.device)
        fl = torch.empty(B, dtype=torch.uint8, device=self.device)
        ws, nb = self.workspace(OP_MH, B)
        check(self.lib.qmc_mh_steps(self.h, B, int(steps), float(stddev), int(seed), int(counter), ptr(e),
                                    ptr(log_prob), ptr(accepts), ptr(normals), ptr(uniforms), ptr(fl),
                                    ptr(ws), ws.numel(), stream_handle(stream)))
        return e, log_prob, accepts, fl

    def mh_steps_resident(self, electrons, steps, stddev, seed, counter, log_prob, accepts, flags=None,
                          ws=None, stream=None):
        """MH updates with the Philox counter in device memory (uint64 tensor of
        one element, advanced by ``steps``); no host synchronisation."""
        e = self._elec(electrons)
        B = e.shape[0]
        if counter.dtype != torch.uint64 and counter.dtype != torch.int64:
            raise ValueError("counter must be a one-element 64-bit integer CUDA tensor")
        if ws is None:
            ws, _ = self.workspace(OP_MH, B)
        check(self.lib.qmc_mh_steps_resident(self.h, B, int(steps), float(stddev), int(seed), ptr(counter),
                                             ptr(e), ptr(log_prob), ptr(accepts), ptr(flags), ptr(ws),
                                             ws.numel(), stream_handle(stream)))
        return e, log_prob, accepts

    def tangent_rows(self, op: int) -> int:
        """Rows per electron that ``op`` propagates (padded tangents for E_L)."""
        return int(self.lib.qmc_tangent_rows(self.h, int(op)))

    def set_grad_budget(self, nbytes: int):
        check(self.lib.qmc_model_set_grad_budget(self.h, int(nbytes)))

    def set_energy_budget(self, nbytes: int):
        """Workspace budget of the chunked Psiformer local energy."""
        check(self.lib.qmc_model_set_energy_budget(self.h, int(nbytes)))

    def grad(self, electrons, weights=None, per_walker=False, stream=None):
        """Adjoint of log|psi|: returns ``(per_walker (B,P) or None, grad (P,) float64 or
        None, logpsi (B,))``; ``grad = sum_w weights[w] d log|psi_w|/d theta``."""
        e = self._elec(electrons)
        B = e.shape[0]
        P = self.param_count
        J = torch.empty((B, P), dtype=torch.float32, device=self.device) if per_walker else None
        g = None
        w = None
        if weights is not None:
            w = weights.to(device=self.device, dtype=torch.float64).contiguous()
            g = torch.empty(P, dtype=torch.float64, device=self.device)
        lp = torch.empty(B, dtype=torch.float32, device=self.device)
        ws, nb = self.workspace(OP_GRAD, B)
        check(self.lib.qmc_grad(self.h, B, ptr(e), ptr(w), ptr(J), ptr(g), ptr(lp), ptr(ws), ws.numel(),
                                stream_handle(stream)))
        return J, g, lp

    def layer_taps(self, electrons, stream=None):
        """Per-layer KFAC statistics of the adjoint (``qmc_grad_taps``): a list
        of dicts with ``kind`` ("dense" or "diagonal"), ``rows_per_walker``,
        ``has_bias``, ``kernel_offset`` / ``bias_offset`` (flat parameter
        offsets), ``x`` (B*rows, in_cols) inputs and ``dy`` (B*rows, out_cols)
        output cotangents of log|psi_w| (for the diagonal tap: per-walker
        gradients of its parameters); plus log|psi| (B,)."""
        e = self._elec(electrons)
        B = e.shape[0]
        n = int(self.lib.qmc_layer_taps(self.h, B, None, 0, None))
        if n < 0:
            raise QmcError(7, "qmc_layer_taps rejected this model")
        descs = (LayerTapC * n)()
        total = C.c_size_t()
        self.lib.qmc_layer_taps(self.h, B, descs, n, C.byref(total))
        buf = torch.empty(int(total.value), dtype=torch.float32, device=self.device)
        lp = torch.empty(B, dtype=torch.float32, device=self.device)
        ws, nb = self.workspace(OP_GRAD, B)
        check(self.lib.qmc_grad_taps(self.h, B, ptr(e), ptr(buf), buf.numel(), ptr(lp), ptr(ws), ws.numel(),
                                     stream_handle(stream)))
        out = []
        for t in descs:
            rows = B * t.rows_per_walker
            x = buf[t.in_offset:t.in_offset + rows * t.in_cols].view(rows, t.in_cols)
            dy = buf[t.out_offset:t.out_offset + rows * t.out_cols].view(rows, t.out_cols)
            out.append({"kind": "dense" if t.kind == TAP_DENSE else "diagonal",
                        "rows_per_walker": t.rows_per_walker, "has_bias": bool(t.has_bias),
                        "kernel_offset": int(t.kernel_offset), "bias_offset": int(t.bias_offset),
                        "in_cols": t.in_cols, "out_cols": t.out_cols, "x": x, "dy": dy})
        return out, lp

    def ecp_energy(self, electrons, tables, rotations=None, seed=0, counter=0, stream=None):
        """ECP energy per walker (``qmc_ecp_energy``): ``(local, nonlocal)``.
        ``tables`` is the dict ECPTables.device() returns (device arrays and
        sizes); ``rotations`` (B, n, 3, 3) or None for Philox draws."""
        e = self._elec(electrons)
        B = e.shape[0]
        t = tables
        loc = torch.empty(B, dtype=torch.float32, device=self.device)
        nl = torch.empty(B, dtype=torch.float32, device=self.device)
        nb = int(self.lib.qmc_ecp_workspace_size(self.h, B, t["n_channels"], t["max_core"], t["n_quad"]))
        ws = self.ws.get(nb)
        rot = None
        if rotations is not None:
            rot = rotations.to(device=self.device, dtype=torch.float32).contiguous()
        check(self.lib.qmc_ecp_energy(self.h, B, ptr(e), t["n_ecp_atoms"], ptr(t["ecp_atoms"]), t["n_channels"],
                                      t["max_terms"], ptr(t["radial"]), t["max_core"], t["n_quad"], ptr(t["quad"]),
                                      ptr(rot), int(seed), int(counter), ptr(loc), ptr(nl), ptr(ws), ws.numel(),
                                      stream_handle(stream)))
        return loc, nl

    def mh_draws(self, batch, steps, seed, counter, stream=None):
        nz = torch.empty((steps, batch, self.n, 3), dtype=torch.float32, device=self.device)
        uz = torch.empty((steps, batch), dtype=torch.float32, device=self.device)
        check(self.lib.qmc_mh_draws(self.h, int(batch), int(steps), int(seed), int(counter), ptr(nz),
                                    ptr(uz), stream_handle(stream)))
        return nz, uz


class NativePsiformer(NativeFermiNet):
    """A ``qmc_model`` handle for a Psiformer (+ SimpleEE Jastrow): the value
    path (``forward``, ``mh_steps``, ``mh_steps_resident``, ``mh_draws``) and
    the forward-Laplacian ``local_energy`` and the FP32 parameter adjoint ``grad``."""

    def __init__(self, cfg, atoms, charges, precision="mixed", device=None):
        self._open(device)
        c = PsiformerConfigC()
        c.n_up, c.n_down = int(cfg.nspins[0]), int(cfg.nspins[1])
        atoms = np.ascontiguousarray(np.asarray(atoms, np.float32).reshape(-1, 3))
        charges = np.ascontiguousarray(np.asarray(charges, np.float32).reshape(-1))
        c.n_atoms = atoms.shape[0]
        c.ndets = int(cfg.ndets)
        c.n_layers = int(cfg.num_layers)
        c.n_heads = int(cfg.num_heads)
        c.head_dim = int(cfg.heads_dim)
        c.n_mlp = len(cfg.mlp_hidden_dims)
        for k, v in enumerate(cfg.mlp_hidden_dims):
            c.mlp_dims[k] = int(v)
        c.envelope = ENVELOPE[str(cfg.envelope)]
        c.orbitals_spin_split = int(bool(cfg.orbitals_spin_split))
        c.jastrow = 1 if cfg.jastrow == "simple_ee" else 0
        c.precision = PRECISION[precision]
        h = C.c_void_p()
        check(self.lib.qmc_psiformer_create(C.byref(c), atoms.ctypes.data, charges.ctypes.data, C.byref(h)))
        self._finish(h, c.n_up + c.n_down, precision)


class NativeLapNet(NativeFermiNet):
    """A ``qmc_model`` handle for LapNet (+ SimpleEE Jastrow): the value path
    (``forward``, ``mh_steps``, ``mh_steps_resident``, ``mh_draws``), the
    forward-Laplacian ``local_energy``, ``ecp_energy`` and the FP32 parameter
    adjoint ``grad``."""

    def __init__(self, cfg, atoms, charges, precision="mixed", device=None):
        if getattr(cfg, "use_layernorm", False):
            raise NotImplementedError("LapNet with use_layernorm=True is not supported")
        self._open(device)
        c = LapNetConfigC()
        c.n_up, c.n_down = int(cfg.nspins[0]), int(cfg.nspins[1])
        atoms = np.ascontiguousarray(np.asarray(atoms, np.float32).reshape(-1, 3))
        charges = np.ascontiguousarray(np.asarray(charges, np.float32).reshape(-1))
        c.n_atoms = atoms.shape[0]
        c.ndets = int(cfg.ndets)
        c.n_layers = int(cfg.num_layers)
        c.n_heads = int(cfg.num_heads)
        c.head_dim = int(cfg.heads_dim)
        c.num_local_updates = int(cfg.num_local_updates)
        c.use_input_bias = int(bool(cfg.use_input_bias))
        c.use_backbone_bias = int(bool(cfg.use_backbone_bias))
        c.envelope = ENVELOPE[str(cfg.envelope)]
        c.orbitals_spin_split = int(bool(getattr(cfg, "orbitals_spin_split", True)))
        c.jastrow = 1 if cfg.jastrow == "simple_ee" else 0
        c.precision = PRECISION[precision]
        h = C.c_void_p()
        check(self.lib.qmc_lapnet_create(C.byref(c), atoms.ctypes.data, charges.ctypes.data, C.byref(h)))
        self._finish(h, c.n_up + c.n_down, precision)


KERNEL_CLASSES = ["stream_layer", "broadcast", "orbital", "logdet", "features", "means", "pair", "mh",
                  "other", "layer0"]


def profile_enable(on: bool = True):
    check(load().qmc_profile_enable(int(bool(on))))


def profile_read():
    """``{class: (launches, ms)}`` since the last read (synchronises)."""
    n = len(KERNEL_CLASSES)
    launches = (C.c_int64 * n)()
    ms = (C.c_double * n)()
    check(load().qmc_profile_read(n, launches, ms))
    return {k: (int(launches[i]), float(ms[i])) for i, k in enumerate(KERNEL_CLASSES)}


class RequestGraph:
    """One VMC request on a resident walker batch -- ``steps`` all-electron MH
    updates with the Philox counter in device memory, the forward-Laplacian
    local energy and its FP64 batch mean and variance (``qmc_mh_steps_resident``
    + ``qmc_local_energy`` + ``qmc_reduce_mean_var``, the reference's
    ``MCMCSampler.step`` + energy estimators + ``mean_reduce``) -- captured
    into a CUDA graph and replayed by :meth:`run`, so the hundreds of launches
    of a request leave the host as one.

    ``electrons`` (B, n, 3) is updated in place by every run; ``counter``
    advances by ``steps`` per run, so runs draw the same Philox stream as
    successive ``mh_steps`` calls from that counter.  Construction runs one
    request eagerly (the library sets per-kernel attributes on first use),
    which advances the walkers and the counter, and then captures, without
    running, the request that :meth:`run` replays."""

    def __init__(self, model, electrons, steps, stddev, seed, counter=0):
        e = model._elec(electrons)
        B = e.shape[0]
        dev = e.device
        self.model, self.electrons, self.steps = model, e, int(steps)
        self.stddev, self.seed = float(stddev), int(seed)
        lib = model.lib
        self.ws_bytes = max(int(lib.qmc_workspace_size(model.h, OP_MH, B)),
                            int(lib.qmc_workspace_size(model.h, OP_LOCAL_ENERGY, B)))
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=dev)
        self.log_prob = torch.empty(B, dtype=torch.float32, device=dev)
        self.accepts = torch.zeros(B, dtype=torch.int32, device=dev)
        self.e_local = torch.empty(B, dtype=torch.float32, device=dev)
        self.mean_var = torch.empty(2, dtype=torch.float64, device=dev)
        self.counter = torch.tensor([int(counter)], dtype=torch.int64, device=dev)
        self.device = dev
        # eager run and capture on a side stream (capture cannot use the
        # legacy default stream), ordered after the caller's pending work
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        self._st = side
        with torch.cuda.stream(side):
            self._enqueue()
        side.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.stream(side):
            self.graph.capture_begin(capture_error_mode="thread_local")
            try:
                self._enqueue()
            finally:
                self.graph.capture_end()

    def _enqueue(self):
        m, lib, st = self.model, self.model.lib, int(self._st.cuda_stream)
        B = self.electrons.shape[0]
        check(lib.qmc_mh_steps_resident(m.h, B, self.steps, self.stddev, self.seed, ptr(self.counter),
                                        ptr(self.electrons), ptr(self.log_prob), ptr(self.accepts), None,
                                        ptr(self.ws), self.ws_bytes, st))
        check(lib.qmc_local_energy(m.h, B, ptr(self.electrons), ptr(self.e_local), None, None, None, None,
                                   ptr(self.ws), self.ws_bytes, st))
        check(lib.qmc_reduce_mean_var(B, ptr(self.e_local), ptr(self.mean_var), st))

    def run(self, stream=None):
        """Replay the request on ``stream`` (default: the current stream), in
        order with the caller's other work there; returns the device tensor
        (E_L mean, variance)."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.stream(s):
            self.graph.replay()
        return self.mean_var


def reduce_mean_var(x: torch.Tensor, stream=None):
    out = torch.empty(2, dtype=torch.float64, device=x.device)
    x = x.to(torch.float32).contiguous()
    check(load().qmc_reduce_mean_var(x.numel(), ptr(x), ptr(out), stream_handle(stream)))
    return out


def warp_mma_peak(device=None, iters=4096, repeats=5):
    """Measured warp-level BF16 MMA (mma.m16n8k16) throughput in TFLOP/s: the
    best of ``repeats`` launches of the library's MMA probe (4 blocks of 8
    warps per SM), timed with CUDA events on the launching stream."""
    dev = torch.device(device or "cuda")
    props = torch.cuda.get_device_properties(dev)
    blocks = props.multi_processor_count * 4
    out = torch.empty(blocks * 256, dtype=torch.float32, device=dev)
    flop = C.c_double()
    lib = load()
    s = torch.cuda.current_stream(dev)
    check(lib.qmc_mma_throughput(blocks, iters, ptr(out), C.byref(flop), stream_handle(s)))
    best = float("inf")
    for _ in range(repeats):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(s)
        check(lib.qmc_mma_throughput(blocks, iters, ptr(out), C.byref(flop), stream_handle(s)))
        e1.record(s)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return flop.value / best / 1e12


def fp32_simt_peak(device=None, iters=4096, repeats=5):
    """Measured FP32 SIMT throughput in TFLOP/s (2 FLOPs per FMA): the best of
    ``repeats`` launches of the library's FMA probe, timed with CUDA events on
    the launching stream after one warm-up launch."""
    dev = torch.device(device or "cuda")
    props = torch.cuda.get_device_properties(dev)
    blocks = props.multi_processor_count * 8
    out = torch.empty(blocks * 256, dtype=torch.float32, device=dev)
    fma = C.c_double()
    lib = load()
    s = torch.cuda.current_stream(dev)
    check(lib.qmc_ffma_throughput(blocks, iters, ptr(out), C.byref(fma), stream_handle(s)))
    best = float("inf")
    for _ in range(repeats):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(s)
        check(lib.qmc_ffma_throughput(blocks, iters, ptr(out), C.byref(fma), stream_handle(s)))
        e1.record(s)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2.0 * fma.value / best / 1e12
