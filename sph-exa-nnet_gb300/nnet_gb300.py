"""Python host side of the GB300 burn library, over its C ABI (include/nnet_gb300.h).

Mirrors the reference's plugin surface for the burn path:

  compute_nuclear_reactions(n, first, last, hydro_dt, previous_dt, reactions, rates, eos,
                            use_drhodt)   <->   nnet::parallel::computeNuclearReactions<true>
                                               (include/nnet/parallel/parallel_nuclear_net.hpp:86-172)
  compute_helm_eos(n, first, last, Z)    <->   nnet::parallel::computeHelmEOS<true>
                                               (parallel_nuclear_net.hpp:191-231)

`n` is any object with the SPH-EXA particle fields the reference requires
(parallel_nuclear_net.hpp:63-85): `Y` (one 1-D CUDA tensor per species), `temp`, `rho`,
`rho_m1`, `dt`, and for the EOS `u`, `cv`, `p`, `c`, `dpdT`.  Networks and EOSes are
passed as the tags below instead of the reference's polymorphic functors.  PyTorch is used
only for device memory and streams; every computation runs in the library's CUDA kernels,
and every call fails loudly when the library or a GPU is missing.
"""
import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnnet_gb300.so")
HELM_TABLE_PATH = os.path.join(HERE, "data", "helm_table.bin")

NET14, NET86, NET87 = 14, 86, 87
EOS_IDEAL_GAS, EOS_HELMHOLTZ = 0, 1
SOLVER_DENSE_FP64, SOLVER_SPARSE_FP64, SOLVER_MIXED = 0, 1, 2
LAYOUT_AUTO, LAYOUT_THREAD, LAYOUT_WARP, LAYOUT_BATCHED = 0, 1, 2, 3
LAYOUTS = {"auto": LAYOUT_AUTO, "thread": LAYOUT_THREAD, "warp": LAYOUT_WARP, "batched": LAYOUT_BATCHED}
STATUS_NAMES = ["OK", "SKIPPED", "LIVELOCK", "MAXITER", "ZERO_DT", "ABORTED"]
ERR_ABORTED = -6
NUM_REACTIONS = {14: 29, 86: 309, 87: 311}
SOLVERS = {"dense": SOLVER_DENSE_FP64, "plain": SOLVER_DENSE_FP64, "sparse": SOLVER_SPARSE_FP64,
           "mixed": SOLVER_MIXED}


class NnetError(RuntimeError):
    pass


class _BurnArgs(ctypes.Structure):
    _fields_ = [("network", ctypes.c_int), ("eos", ctypes.c_int), ("ideal_gas_mu", ctypes.c_double),
                ("solver", ctypes.c_int), ("num_particles", ctypes.c_size_t),
                ("Y", ctypes.POINTER(ctypes.c_void_p)), ("T", ctypes.c_void_p), ("rho", ctypes.c_void_p),
                ("rho_m1", ctypes.c_void_p), ("dt", ctypes.c_void_p), ("hydro_dt", ctypes.c_double),
                ("previous_dt", ctypes.c_double), ("use_drhodt", ctypes.c_int),
                ("max_newton_iterations", ctypes.c_longlong), ("status", ctypes.c_void_p),
                ("substeps", ctypes.c_void_p), ("iterations", ctypes.c_void_p),
                ("time_limit_seconds", ctypes.c_double), ("normalize_mass", ctypes.c_int),
                ("mass_drift", ctypes.c_void_p), ("u", ctypes.c_void_p), ("cv", ctypes.c_void_p),
                ("p", ctypes.c_void_p), ("c", ctypes.c_void_p), ("dpdT", ctypes.c_void_p),
                ("order", ctypes.c_void_p)]


class _Stats(ctypes.Structure):
    _fields_ = [("newton_iterations", ctypes.c_ulonglong), ("substeps", ctypes.c_ulonglong),
                ("status_count", ctypes.c_ulonglong * len(STATUS_NAMES)), ("refinement_steps", ctypes.c_ulonglong),
                ("fp64_fallbacks", ctypes.c_ulonglong)]


def _dptr(t):
    return None if t is None else t.data_ptr()


def burn_args(network, Y, T, rho, dt, hydro_dt, eos=EOS_HELMHOLTZ, mu=0.0, rho_m1=None, previous_dt=0.0,
              use_drhodt=False, solver=SOLVER_DENSE_FP64, max_iter=100000, status=None, substeps=None,
              iterations=None, time_limit=0.0, normalize_mass=False, mass_drift=None, eos_out=None, order=None):
    """The nnet_burn_args of a burn (CUDA tensors; Y a list of per-species tensors or a 2-D
    [species, particles] tensor).  Returns (args, keep): `keep` holds the pointer array the
    arguments refer to and must outlive the call.  eos_out: None or the five tensors
    (u, cv, p, c, dpdT) of the post-burn Helmholtz EOS; order: None or an int32 CUDA tensor
    holding a permutation of the particle indices (the work queue's visiting order)."""
    import torch
    if isinstance(solver, str):
        solver = SOLVERS[solver]
    if isinstance(eos, str):
        eos = EOS_IDEAL_GAS if eos.startswith("ideal") else EOS_HELMHOLTZ
    rows = [Y[j] for j in range(network)]
    outs = list(eos_out) if eos_out is not None else [None] * 5
    if len(outs) != 5:
        raise NnetError("eos_out needs the five tensors u, cv, p, c, dpdT")
    named = [("T", T), ("rho", rho), ("dt", dt), ("rho_m1", rho_m1), ("mass_drift", mass_drift)]
    named += [("Y", r) for r in rows] + list(zip(["u", "cv", "p", "c", "dpdT"], outs))
    for name, t in named:
        _require_cuda(t, name)
        if t is not None and t.dtype != torch.float64:
            raise NnetError(f"{name} must be float64")
        # the library reads every array (and every species row of Y) as densely packed
        if t is not None and t.dim() == 1 and t.numel() > 1 and t.stride(0) != 1:
            raise NnetError(f"{name} must be contiguous (got stride {t.stride(0)})")
    if order is not None and (order.dtype != torch.int32 or order.numel() != T.numel() or not order.is_cuda):
        raise NnetError("order must be an int32 CUDA tensor of num_particles indices")
    yp = (ctypes.c_void_p * network)(*[r.data_ptr() for r in rows])
    a = _BurnArgs(network=network, eos=eos, ideal_gas_mu=mu, solver=solver, num_particles=T.numel(),
                  Y=ctypes.cast(yp, ctypes.POINTER(ctypes.c_void_p)), T=T.data_ptr(), rho=rho.data_ptr(),
                  rho_m1=_dptr(rho_m1), dt=dt.data_ptr(), hydro_dt=hydro_dt, previous_dt=previous_dt,
                  use_drhodt=int(bool(use_drhodt)), max_newton_iterations=max_iter, status=_dptr(status),
                  substeps=_dptr(substeps), iterations=_dptr(iterations), time_limit_seconds=time_limit,
                  normalize_mass=int(bool(normalize_mass)), mass_drift=_dptr(mass_drift), u=_dptr(outs[0]),
                  cv=_dptr(outs[1]), p=_dptr(outs[2]), c=_dptr(outs[3]), dpdT=_dptr(outs[4]), order=_dptr(order))
    return a, yp


_lib = None


def load_library(path=LIB_PATH):
    """Load libnnet_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise NnetError(f"{path} is missing: build it with __graft_entry__.build() or sph-exa-nnet_gb300/nnet_build.py")
    lib = ctypes.CDLL(path)
    P, I, S, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_double
    lib.nnet_create.argtypes = [I, ctypes.POINTER(P)]
    lib.nnet_destroy.argtypes = [P]
    lib.nnet_load_helmholtz_table.argtypes = [P, P]
    lib.nnet_load_helmholtz_table_file.argtypes = [P, ctypes.c_char_p]
    lib.nnet_burn.argtypes = [P, ctypes.POINTER(_BurnArgs), P]
    lib.nnet_get_stats.argtypes = [P, ctypes.POINTER(_Stats)]
    lib.nnet_helmholtz_eos.argtypes = [P, S, I, P, P, P, P, P, P, P, P, P, P]
    lib.nnet_network_info.argtypes = [I, ctypes.POINTER(I), ctypes.POINTER(I)]
    lib.nnet_last_error_message.restype = ctypes.c_char_p
    lib.nnet_solver_info.argtypes = [I, I, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                                     ctypes.POINTER(I)]
    lib.nnet_measure_fp64_peak.argtypes = [I, ctypes.POINTER(D)]
    lib.nnet_set_layout.argtypes = [P, I]
    lib.nnet_set_batch_slots.argtypes = [P, I]
    lib.nnet_burn_batch.argtypes = [P, ctypes.POINTER(_BurnArgs), I, P]
    lib.nnet_burn_noalloc.argtypes = [P, ctypes.POINTER(_BurnArgs), P]
    lib.nnet_cost_order.argtypes = [P, S, P, P, P]
    lib.nnet_set_rebalance.argtypes = [P, I]
    _lib = lib
    return lib


def _check(rc):
    if rc != 0:
        raise NnetError(f"nnet error {rc}: {_lib.nnet_last_error_message().decode()}")


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _require_cuda(t, name):
    if t is not None and not t.is_cuda:
        raise NnetError(f"{name} must be a CUDA tensor (the library has no CPU path)")


def _require_dense(t, name):
    if t is not None and t.numel() > 1 and not t.is_contiguous():
        raise NnetError(f"{name} must be contiguous")


class Context:
    """One library context (per device): network tables resident in HBM, optional
    Helmholtz table, and the persistent-kernel scratch."""

    def __init__(self, device=0, helmholtz_table=HELM_TABLE_PATH):
        import torch
        if not torch.cuda.is_available():
            raise NnetError("no CUDA device: the GB300 burn library has no CPU fallback")
        lib = load_library()
        self.device = device
        h = ctypes.c_void_p()
        _check(lib.nnet_create(device, ctypes.byref(h)))
        self.handle = h
        if helmholtz_table is not None:
            self.load_helmholtz_table(helmholtz_table)

    def set_layout(self, layout):
        """Particle layout of the sparse / mixed solvers: "auto", "thread", "warp" or "batched"."""
        _check(_lib.nnet_set_layout(self.handle, LAYOUTS[layout] if isinstance(layout, str) else int(layout)))

    def set_rebalance(self, on):
        """Batched layout: hand running particles between warps once the queue drains (default on)."""
        _check(_lib.nnet_set_rebalance(self.handle, int(bool(on))))

    def set_batch_slots(self, slots):
        """Batched layout: particles in flight per warp (1..32)."""
        _check(_lib.nnet_set_batch_slots(self.handle, int(slots)))

    def close(self):
        if self.handle:
            _lib.nnet_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_helmholtz_table(self, table):
        """`table`: path to the binary stand-in, path to a reference-format text table
        (helm_table.dat), or a float64 array of 21 x 541 x 201 values."""
        if isinstance(table, str):
            if table.endswith(".bin"):
                table = np.fromfile(table, dtype="<f8")
            else:
                _check(_lib.nnet_load_helmholtz_table_file(self.handle, table.encode()))
                return
        table = np.ascontiguousarray(table, dtype=np.float64).reshape(-1)
        if table.size != 21 * 541 * 201:
            raise NnetError("Helmholtz table must hold 21 x 541 x 201 doubles")
        _check(_lib.nnet_load_helmholtz_table(self.handle, table.ctypes.data_as(ctypes.c_void_p)))

    def burn(self, network, Y, T, rho, dt, hydro_dt, eos=EOS_HELMHOLTZ, mu=0.0, rho_m1=None, previous_dt=0.0,
             use_drhodt=False, solver=SOLVER_DENSE_FP64, max_iter=100000, status=None, substeps=None,
             iterations=None, stream=None, time_limit=0.0, normalize_mass=False, mass_drift=None, eos_out=None,
             order=None):
        """Burn in place (nnet_burn).  Y: list of per-species 1-D CUDA float64 tensors (or a 2-D
        [species, particles] tensor); T, dt updated in place.  time_limit: launch watchdog in
        seconds (0: none); normalize_mass / mass_drift / eos_out: the post-burn steps; order: the
        work queue's visiting order."""
        import torch
        a, keep = burn_args(network, Y, T, rho, dt, hydro_dt, eos, mu, rho_m1, previous_dt, use_drhodt, solver,
                            max_iter, status, substeps, iterations, time_limit, normalize_mass, mass_drift, eos_out,
                            order)
        s = torch.cuda.current_stream(self.device) if stream is None else stream
        _check(_lib.nnet_burn(self.handle, ctypes.byref(a), ctypes.c_void_p(s.cuda_stream)))

    def burn_batch(self, batches, solver=SOLVER_SPARSE_FP64, eos=EOS_HELMHOLTZ, mu=0.0, max_iter=100000, stream=None,
                   normalize_mass=False):
        """One launch over sub-batches of different networks (nnet_burn_batch).  `batches`: list of
        dicts with keys network, Y, T, rho, dt, hydro_dt and optional status / iterations /
        substeps / mass_drift / eos_out (CUDA tensors)."""
        import torch
        arr = (_BurnArgs * len(batches))()
        keep = []
        for k, b in enumerate(batches):
            a, yp = burn_args(b["network"], b["Y"], b["T"], b["rho"], b["dt"], b["hydro_dt"], eos, mu, solver=solver,
                              max_iter=max_iter, status=b.get("status"), substeps=b.get("substeps"),
                              iterations=b.get("iterations"), normalize_mass=normalize_mass,
                              mass_drift=b.get("mass_drift"), eos_out=b.get("eos_out"))
            arr[k] = a
            keep.append(yp)
        s = torch.cuda.current_stream(self.device) if stream is None else stream
        _check(_lib.nnet_burn_batch(self.handle, arr, len(batches), ctypes.c_void_p(s.cuda_stream)))

    def burn_noalloc(self, network, Y, T, rho, dt, hydro_dt, stream=None, **kw):
        """nnet_burn_noalloc: the batched-layout burn with the library's fixed scratch arrays
        (no device allocation); same keywords as burn (sparse and mixed solvers only)."""
        import torch
        a, keep = burn_args(network, Y, T, rho, dt, hydro_dt, **kw)
        s = torch.cuda.current_stream(self.device) if stream is None else stream
        _check(_lib.nnet_burn_noalloc(self.handle, ctypes.byref(a), ctypes.c_void_p(s.cuda_stream)))

    def cost_order(self, cost, stream=None):
        """nnet_cost_order: an int32 CUDA tensor holding a permutation of the particles with the
        costliest first (decreasing power-of-two class of `cost`, an int32 CUDA tensor such as a
        previous burn's iterations), for burn(order=...)."""
        import torch
        if cost.dtype != torch.int32 or not cost.is_cuda:
            raise NnetError("cost must be an int32 CUDA tensor")
        order = torch.empty_like(cost)
        s = torch.cuda.current_stream(self.device) if stream is None else stream
        _check(_lib.nnet_cost_order(self.handle, cost.numel(), _ptr(cost), _ptr(order), ctypes.c_void_p(s.cuda_stream)))
        return order

    def stats(self):
        """Statistics of the last burn on this context; `aborted` is True when that launch
        stopped at its time limit (nnet_get_stats returned NNET_ERR_ABORTED)."""
        st = _Stats()
        rc = _lib.nnet_get_stats(self.handle, ctypes.byref(st))
        if rc not in (0, ERR_ABORTED):
            _check(rc)
        return dict(newton_iterations=st.newton_iterations, substeps=st.substeps,
                    status=dict(zip(STATUS_NAMES, list(st.status_count))), refinement_steps=st.refinement_steps,
                    fp64_fallbacks=st.fp64_fallbacks, aborted=rc == ERR_ABORTED)

    def helmholtz_eos(self, Z, T, rho, Y, u, cv, p, c, dpdT, stream=None):
        import torch
        Z = np.ascontiguousarray(Z, dtype=np.float64)
        rows = [Y[j] for j in range(Z.size)]
        for name, t in [("T", T), ("rho", rho), ("u", u), ("cv", cv), ("p", p), ("c", c), ("dpdT", dpdT)] + [
                ("Y", r) for r in rows]:
            _require_cuda(t, name)
            _require_dense(t, name)
        yp = (ctypes.c_void_p * Z.size)(*[r.data_ptr() for r in rows])
        s = torch.cuda.current_stream(self.device) if stream is None else stream
        _check(_lib.nnet_helmholtz_eos(self.handle, T.numel(), Z.size, Z.ctypes.data_as(ctypes.c_void_p),
                                       _ptr(T), _ptr(rho), ctypes.cast(yp, ctypes.c_void_p), _ptr(u), _ptr(cv),
                                       _ptr(p), _ptr(c), _ptr(dpdT), ctypes.c_void_p(s.cuda_stream)))


# ---------------------------------------------------------------- reference-shaped API
@dataclass(frozen=True)
class ReactionList:
    """Tag standing in for nnet::netXX::reactionList."""
    network: int


@dataclass(frozen=True)
class ComputeReactionRates:
    """Tag standing in for nnet::netXX::computeReactionRates."""
    network: int


@dataclass(frozen=True)
class IdealGasFunctor:
    """nnet::eos::IdealGasFunctor(mu) (ideal_gas.hpp:46-83)."""
    mu: float


@dataclass(frozen=True)
class HelmholtzFunctor:
    """nnet::eos::HelmholtzFunctor over the network's charges (helmholtz.hpp:150-226)."""
    network: int = 86


net14_reactionList, net14_computeReactionRates = ReactionList(14), ComputeReactionRates(14)
net86_reactionList, net86_computeReactionRates = ReactionList(86), ComputeReactionRates(86)
net87_reactionList, net87_computeReactionRates = ReactionList(87), ComputeReactionRates(87)

_default_context = {}


def default_context(device=0):
    if device not in _default_context:
        _default_context[device] = Context(device)
    return _default_context[device]


def compute_nuclear_reactions(n, first, last, hydro_dt, previous_dt, reactions, construct_rates_BE, eos,
                              use_drhodt=False, solver=SOLVER_SPARSE_FP64, context=None, status=None,
                              max_iter=100000):
    """Burn particles [first, last) of `n` over hydro_dt, in place (Y, temp, dt), on the
    current CUDA stream.  Same parameters as computeNuclearReactions
    (parallel_nuclear_net.hpp:86-90); `solver` selects the linear-solve form."""
    if reactions.network != construct_rates_BE.network:
        raise NnetError("reaction list and rate functor belong to different networks")
    net = reactions.network
    if len(n.Y) != net:
        raise NnetError(f"data holds {len(n.Y)} species, network {net} needs {net}")
    ctx = context or default_context(n.temp.device.index or 0)
    sl = slice(first, last)
    rho_m1 = getattr(n, "rho_m1", None)
    if use_drhodt and rho_m1 is None:
        use_drhodt = False  # as the reference when rho_m1 is not allocated (parallel_nuclear_net.hpp:103-114)
    kw = dict(eos=EOS_IDEAL_GAS, mu=eos.mu) if isinstance(eos, IdealGasFunctor) else dict(eos=EOS_HELMHOLTZ)
    ctx.burn(net, [y[sl] for y in n.Y], n.temp[sl], n.rho[sl], n.dt[sl], hydro_dt,
             rho_m1=None if rho_m1 is None else rho_m1[sl], previous_dt=previous_dt, use_drhodt=use_drhodt,
             solver=solver, status=None if status is None else status[sl], max_iter=max_iter, **kw)


def solver_info(network, solver):
    """(factorisation FMAs, triangular-solve FMAs, stored factor entries) of one Newton solve."""
    lib = load_library()
    if isinstance(solver, str):
        solver = SOLVERS[solver]
    f, s, e = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_int()
    _check(lib.nnet_solver_info(network, solver, ctypes.byref(f), ctypes.byref(s), ctypes.byref(e)))
    return f.value, s.value, e.value


def measure_fp64_peak(device=0):
    """FP64 FMA throughput of the device in TFLOP/s (dependency-free probe kernel)."""
    lib = load_library()
    t = ctypes.c_double()
    _check(lib.nnet_measure_fp64_peak(device, ctypes.byref(t)))
    return t.value


def network_charges(network):
    """Z of a network's species (net87 includes the electron entry, Z = -1)."""
    import re
    src = open(os.path.join(HERE, "data", "nnet_network_tables.h")).read()
    name = "net14_Z" if network == 14 else "net86_Z"
    body = re.search(name + r"\[\d+\] = \{([^}]*)\}", src).group(1)
    return np.array([float(v) for v in body.split(",")])[:network]


def compute_helm_eos(n, first, last, Z, context=None):
    """Post-burn Helmholtz EOS into n.u, n.cv, n.p, n.c, n.dpdT for [first, last)
    (computeHelmEOS, parallel_nuclear_net.hpp:191-261)."""
    ctx = context or default_context(n.temp.device.index or 0)
    sl = slice(first, last)
    ctx.helmholtz_eos(Z, n.temp[sl], n.rho[sl], [y[sl] for y in n.Y], n.u[sl], n.cv[sl], n.p[sl], n.c[sl],
                      n.dpdT[sl])


# ---------------------------------------------------------------- burn server
class _ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_double), ("solver", ctypes.c_int),
                ("slice_iterations", ctypes.c_longlong), ("max_concurrent_requests", ctypes.c_int)]


class _Request(ctypes.Structure):
    _fields_ = [("network", ctypes.c_int), ("eos", ctypes.c_int), ("ideal_gas_mu", ctypes.c_double),
                ("num_particles", ctypes.c_size_t), ("Y", ctypes.c_void_p), ("T", ctypes.c_void_p),
                ("rho", ctypes.c_void_p), ("dt", ctypes.c_void_p), ("status", ctypes.c_void_p),
                ("hydro_dt", ctypes.c_double), ("max_newton_iterations", ctypes.c_longlong)]


class _ServerStats(ctypes.Structure):
    _fields_ = [("completed_requests", ctypes.c_ulonglong), ("completed_particles", ctypes.c_double),
                ("span_seconds", ctypes.c_double), ("latency_p50", ctypes.c_double),
                ("latency_p95", ctypes.c_double), ("latency_p99", ctypes.c_double),
                ("latency_max", ctypes.c_double), ("slices", ctypes.c_ulonglong)]


class Server:
    """Continuous-batching burn server over the C ABI (nnet_server_*).  Requests carry
    host numpy arrays (float64; Y species-major [network, P]); results overwrite them."""

    def __init__(self, context, solver=SOLVER_SPARSE_FP64, hbm_budget_bytes=150e9, slice_iterations=64,
                 max_concurrent_requests=8):
        lib = load_library()
        P = ctypes.c_void_p
        lib.nnet_server_create.argtypes = [P, ctypes.POINTER(_ServerConfig), ctypes.POINTER(P)]
        lib.nnet_server_submit.argtypes = [P, ctypes.POINTER(_Request), ctypes.POINTER(ctypes.c_uint64)]
        lib.nnet_server_query.argtypes = [P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int)]
        lib.nnet_server_wait.argtypes = [P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double)]
        lib.nnet_server_get_stats.argtypes = [P, ctypes.POINTER(_ServerStats)]
        lib.nnet_server_destroy.argtypes = [P]
        if isinstance(solver, str):
            solver = SOLVERS[solver]
        cfg = _ServerConfig(hbm_budget_bytes, solver, slice_iterations, max_concurrent_requests)
        s = ctypes.c_void_p()
        rc = lib.nnet_server_create(context.handle, ctypes.byref(cfg), ctypes.byref(s))
        if rc != 0:
            raise NnetError(f"nnet_server_create failed ({rc})")
        self.handle, self.context, self._keep = s, context, {}

    def submit(self, network, Y, T, rho, dt, hydro_dt, eos=EOS_HELMHOLTZ, mu=0.0, status=None, max_iter=100000):
        if isinstance(eos, str):
            eos = EOS_IDEAL_GAS if eos.startswith("ideal") else EOS_HELMHOLTZ
        for a in (Y, T, rho, dt):
            if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
                raise NnetError("request arrays must be C-contiguous float64")
        r = _Request(network, eos, mu, T.size, Y.ctypes.data, T.ctypes.data, rho.ctypes.data, dt.ctypes.data,
                     None if status is None else status.ctypes.data, hydro_dt, max_iter)
        rid = ctypes.c_uint64()
        _check(_lib.nnet_server_submit(self.handle, ctypes.byref(r), ctypes.byref(rid)))
        self._keep[rid.value] = (Y, T, rho, dt, status)
        return rid.value

    def done(self, rid):
        d = ctypes.c_int()
        _check(_lib.nnet_server_query(self.handle, rid, ctypes.byref(d)))
        return d.value

    def wait(self, rid):
        lat = ctypes.c_double()
        rc = _lib.nnet_server_wait(self.handle, rid, ctypes.byref(lat))
        self._keep.pop(rid, None)
        if rc != 0:
            raise NnetError(f"request {rid} failed")
        return lat.value

    def stats(self):
        st = _ServerStats()
        _check(_lib.nnet_server_get_stats(self.handle, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _ServerStats._fields_}

    def close(self):
        if self.handle:
            _lib.nnet_server_destroy(self.handle)
            self.handle = None
