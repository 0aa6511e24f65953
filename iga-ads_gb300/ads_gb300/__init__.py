"""Python mirror of the IGA-ADS explicit-step API over the GB300 C-ABI.

The names follow the reference (marcinlos/iga-ads): a :class:`Dimension`
holds what ``ads::dimension`` holds (include/ads/simulation/dimension.hpp:20-59),
:func:`ads_solve` is ``ads::ads_solve`` (include/ads/solver.hpp:222-226),
:class:`Heat` runs ``heat_3d``'s step (examples/heat/heat_3d.hpp:39-67) and
:func:`dgbtrs` is the LAPACK call the reference makes for every direction
(include/ads/lin/band_solve.hpp:20-31).  Every call goes through
``libads_gb300.so`` (include/ads_gb300.h); there is no CPU fallback: if the
library or a GPU is missing, the calls raise.

Device buffers may be given as ``torch`` CUDA tensors (float64, contiguous)
or as raw integer device addresses; host buffers are ``numpy`` float64 arrays.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# ADSG_LIBRARY=checked loads the debug build with device-side bounds checks
# (python iga-ads_gb300/build.py --checked) in place of the release engine.
LIB_PATH = os.path.join(_HERE, "libads_gb300_checked.so" if os.environ.get("ADSG_LIBRARY") == "checked"
                        else "libads_gb300.so")

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_double_p = ctypes.POINTER(ctypes.c_double)


class AdsError(RuntimeError):
    """A non-zero status from the C-ABI (message from adsg_last_error)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"ads_gb300 error {code}: {message}")
        self.code = code


class DimDesc(ctypes.Structure):
    """adsg_dim_desc (include/ads_gb300.h)."""

    _fields_ = [
        ("p", ctypes.c_int),
        ("elements", ctypes.c_int),
        ("quad_order", ctypes.c_int),
        ("n", ctypes.c_int),
        ("btab", _c_double_p),
        ("w", _c_double_p),
        ("J", _c_double_p),
        ("first_dofs", _c_int_p),
        ("kl", ctypes.c_int),
        ("ku", ctypes.c_int),
        ("ldab", ctypes.c_int),
        ("lu", _c_double_p),
        ("ipiv", _c_int_p),
        ("xq", _c_double_p),
    ]


class PointForm(ctypes.Structure):
    """adsg_point_form (include/ads_gb300.h): constants plus optional
    per-Gauss-point fields (device addresses) of A u v + B grad u.grad v + G v + D."""

    _fields_ = [
        ("alpha", ctypes.c_double),
        ("beta", ctypes.c_double),
        ("gamma", ctypes.c_double),
        ("delta", ctypes.c_double),
        ("alpha_q", ctypes.c_void_p),
        ("beta_q", ctypes.c_void_p),
        ("gamma_q", ctypes.c_void_p),
        ("delta_q", ctypes.c_void_p),
    ]


class Plane(ctypes.Structure):
    """adsg_plane: the dofs whose index along direction `dim` is `index`;
    `values` a device address (x-fastest over the other directions) or None
    for zeros."""

    _fields_ = [("dim", ctypes.c_int), ("index", ctypes.c_int), ("values", ctypes.c_void_p)]


def _planes(planes):
    """[(dim, index, values or None), ...] -> a ctypes array of Plane."""
    planes = list(planes)
    arr = (Plane * max(1, len(planes)))()
    for k, (d, idx, vals) in enumerate(planes):
        arr[k].dim, arr[k].index = int(d), int(idx)
        arr[k].values = None if vals is None else _devptr(vals)
    return arr, len(planes)


_lib = None


def library() -> ctypes.CDLL:
    """Load libads_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python iga-ads_gb300/build.py` "
            "(or __graft_entry__.build()); there is no CPU fallback")
    lib = ctypes.CDLL(LIB_PATH)
    vp, i, d, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
    sig = {
        "adsg_dim_create": (i, [i, i, d, d, i, ctypes.POINTER(vp)]),
        "adsg_dim_destroy": (None, [vp]),
        "adsg_dim_describe": (i, [vp, ctypes.POINTER(DimDesc)]),
        "adsg_dim_fix_dof": (i, [vp, i]),
        "adsg_dim_form_band": (i, [vp, i, _c_double_p]),
        "adsg_ctx_create": (i, [i, ctypes.POINTER(DimDesc), ctypes.POINTER(vp)]),
        "adsg_ctx_destroy": (i, [vp]),
        "adsg_ctx_size": (ll, [vp]),
        "adsg_ctx_set_stream": (i, [vp, vp]),
        "adsg_ctx_synchronize": (i, [vp]),
        "adsg_last_error": (ctypes.c_char_p, []),
        "adsg_heat_rhs": (i, [vp, vp, vp, d]),
        "adsg_heat_rhs_elem": (i, [vp, vp, vp, vp, d]),
        "adsg_kappa_points_count": (ll, [vp]),
        "adsg_kappa_points": (i, [vp, vp, vp]),
        "adsg_heat_rhs_elem_points": (i, [vp, vp, vp, vp, d]),
        "adsg_ads_solve": (i, [vp, vp, vp]),
        "adsg_ads_solve_t": (i, [vp, vp]),
        "adsg_heat_step": (i, [vp, vp, vp, d]),
        "adsg_set_planes": (i, [vp, vp, i, ctypes.POINTER(Plane)]),
        "adsg_heat_step_dirichlet": (i, [vp, vp, vp, d, i, ctypes.POINTER(Plane)]),
        "adsg_form_rhs": (i, [vp, vp, ctypes.POINTER(PointForm), vp]),
        "adsg_heat_steps": (i, [vp, vp, d, i]),
        "adsg_heat_steps_host": (i, [vp, _c_double_p, d, i]),
        "adsg_ads_solve_host": (i, [vp, _c_double_p]),
        "adsg_heat_rhs_host": (i, [vp, _c_double_p, _c_double_p, d]),
        "adsg_ctx_enable_stage_timers": (i, [vp, i]),
        "adsg_ctx_stage_times": (i, [vp, _c_double_p, ctypes.POINTER(ctypes.c_longlong)]),
        "adsg_ctx_stage_work": (i, [vp, _c_double_p, _c_double_p]),
        "adsg_ctx_solve_variants": (i, [vp, _c_int_p]),
        "adsg_ctx_step_solve_variants": (i, [vp, _c_int_p]),
        "adsg_ctx_launch_pdl": (i, [vp]),
        "adsg_ctx_fused_x": (i, [vp]),
        "adsg_ctx_step_1block": (i, [vp]),
        "adsg_ctx_step_cluster": (i, [vp]),
        "adsg_ctx_step_graphs": (i, [vp]),
        "adsg_quad_size": (ll, [vp]),
        "adsg_count_nonfinite": (i, [vp, vp, ctypes.POINTER(ll)]),
        "adsg_load_vector": (i, [vp, vp, vp]),
        "adsg_projection": (i, [vp, vp, vp]),
        "adsg_eval_quad": (i, [vp, vp, vp, vp]),
        "adsg_norms": (i, [vp, vp, _c_double_p, _c_double_p]),
        "adsg_errors": (i, [vp, vp, vp, vp, _c_double_p, _c_double_p]),
        "adsg_quad_points": (i, [vp, i, _c_double_p]),
        "adsg_adjoint_create": (i, [vp, i, d, i, ctypes.POINTER(vp)]),
        "adsg_adjoint_destroy": (i, [vp]),
        "adsg_adjoint_checkpoints": (i, [vp, _c_int_p, _c_int_p]),
        "adsg_adjoint_forward": (i, [vp, vp, vp, vp]),
        "adsg_adjoint_backward": (i, [vp, vp, vp, vp]),
        "adsg_mass_loss": (i, [vp, vp, vp, vp, _c_double_p, vp]),
        "adsg_batch_create": (i, [i, _c_int_p, _c_int_p, _c_int_p, _c_double_p, ctypes.POINTER(vp)]),
        "adsg_batch_destroy": (i, [vp]),
        "adsg_batch_dofs": (ll, [vp, i]),
        "adsg_batch_set_state": (i, [vp, i, _c_double_p]),
        "adsg_batch_get_state": (i, [vp, i, _c_double_p]),
        "adsg_batch_steps": (i, [vp, i]),
        "adsg_batch_steps_looped": (i, [vp, i]),
        "adsg_batch_synchronize": (i, [vp]),
        "adsg_batch_tuning": (i, [vp, _c_int_p, _c_int_p]),
        "adsg_batch_engine": (i, [vp]),
        "adsg_batch_order": (i, [vp]),
        "adsg_batch_test_waits": (i, [vp, i, ll]),
        "adsg_test_fail_device_alloc": (i, [i]),
        "adsg_debug_bounds": (i, [ctypes.POINTER(ll), _c_int_p, _c_int_p, ctypes.POINTER(ll), ctypes.POINTER(ll), i]),
        "adsg_dgbtrs_": (i, [ctypes.c_char_p, _c_int_p, _c_int_p, _c_int_p, _c_int_p, _c_double_p, _c_int_p,
                             _c_int_p, _c_double_p, _c_int_p, _c_int_p]),
        "adsg_dgbtrs_checked_": (i, [ctypes.c_char_p, _c_int_p, _c_int_p, _c_int_p, _c_int_p, _c_double_p, _c_int_p,
                                     _c_int_p, _c_double_p, _c_int_p, _c_int_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def debug_bounds(reset: bool = False) -> dict:
    """Out-of-bounds accesses the bounds-checked build's kernels caught (and
    skipped) since the last reset: {"violations", "file", "line", "index",
    "extent"} of the first one.  Raises AdsError in the release build."""
    ll = ctypes.c_longlong
    v, idx, ext = ll(0), ll(0), ll(0)
    f, line = ctypes.c_int(0), ctypes.c_int(0)
    _check(library().adsg_debug_bounds(ctypes.byref(v), ctypes.byref(f), ctypes.byref(line), ctypes.byref(idx),
                                       ctypes.byref(ext), int(reset)))
    files = ("adsg_kernels.cu", "adsg_elem.cu", "adsg_quad.cu")
    return {"violations": v.value, "file": files[f.value] if 0 <= f.value < 3 else None, "line": line.value,
            "index": idx.value, "extent": ext.value}


def test_fail_device_alloc(k: int) -> int:
    """Test hook: the k-th device allocation of the library from now on
    fails as on a full device (ADSG_ERR_NOMEM), then the hook is off; -1 turns
    it off.  Returns the previous setting (-1: no failure was pending)."""
    return int(library().adsg_test_fail_device_alloc(int(k)))


def _check(code: int) -> None:
    if code != 0:
        msg = library().adsg_last_error()
        raise AdsError(code, msg.decode() if msg else "")


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_c_double_p)


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(_c_int_p)


def _devptr(x) -> int:
    """Device address of a torch CUDA float64 tensor (or an int address)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if getattr(x, "is_cuda", False):
        if str(x.dtype) != "torch.float64":
            raise TypeError("device tensors must be float64")
        if not x.is_contiguous():
            raise ValueError("device tensors must be contiguous")
        return x.data_ptr()
    raise TypeError(f"expected a CUDA tensor or a device address, got {type(x)!r}")


def _host(a: np.ndarray) -> np.ndarray:
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
        raise TypeError("host buffers must be C-contiguous float64 numpy arrays")
    return a


NSTAGES = 9
STAGES = ("rhs_outer", "rhs_middle", "rhs_x", "solve_x", "solve_y", "solve_z", "rhs_elem", "rhs_solve_x", "step_1block")


class Dimension:
    """One dimension: open uniform B-spline basis on [a, b], its Gauss tables,
    its mass matrix and that matrix's pivoted band LU (ads::dimension with
    derivatives = 1 after factorize_matrix())."""

    def __init__(self, p: int, elements: int, a: float = 0.0, b: float = 1.0, quad_order: int = 0):
        lib = library()
        h = ctypes.c_void_p()
        _check(lib.adsg_dim_create(p, elements, a, b, quad_order, ctypes.byref(h)))
        self._h = h
        self._desc = DimDesc()
        _check(lib.adsg_dim_describe(h, ctypes.byref(self._desc)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.adsg_dim_destroy(h)
            self._h = None

    @property
    def p(self) -> int:
        return self._desc.p

    @property
    def elements(self) -> int:
        return self._desc.elements

    def dofs(self) -> int:
        return self._desc.n

    @property
    def quad_order(self) -> int:
        return self._desc.quad_order

    def descriptor(self) -> DimDesc:
        return self._desc

    def fix_dof(self, k: int) -> None:
        """dimension::fix_dof: identity row k of M (affects the solve only)."""
        _check(library().adsg_dim_fix_dof(self._h, k))
        _check(library().adsg_dim_describe(self._h, ctypes.byref(self._desc)))

    def fix_left(self) -> None:
        self.fix_dof(0)

    def fix_right(self) -> None:
        self.fix_dof(self.dofs() - 1)

    def form_band(self, which: int) -> np.ndarray:
        """Mass (0) or stiffness (1) band, LAPACK layout kl = ku = p, shape (n, 3p+1)."""
        ldab = 3 * self.p + 1
        out = np.zeros(ldab * self.dofs())
        _check(library().adsg_dim_form_band(self._h, which, _dptr(out)))
        return out.reshape(self.dofs(), ldab)

    def tables(self) -> dict:
        """Copies of the basis_data-like tables and the factorised band."""
        d = self._desc
        nb = d.elements * d.quad_order * 2 * (d.p + 1)
        return {
            "btab": np.ctypeslib.as_array(d.btab, (nb,)).copy(),
            "w": np.ctypeslib.as_array(d.w, (d.quad_order,)).copy(),
            "J": np.ctypeslib.as_array(d.J, (d.elements,)).copy(),
            "first_dofs": np.ctypeslib.as_array(d.first_dofs, (d.elements,)).copy(),
            "lu": np.ctypeslib.as_array(d.lu, (d.ldab * d.n,)).copy(),
            "ipiv": np.ctypeslib.as_array(d.ipiv, (d.n,)).copy(),
            "xq": np.ctypeslib.as_array(d.xq, (d.elements * d.quad_order,)).copy(),
            "kl": d.kl,
            "ku": d.ku,
            "ldab": d.ldab,
        }


class Context:
    """Device-side state for a 1-3D tensor-product space (adsg_ctx)."""

    def __init__(self, dims: Sequence[Dimension]):
        lib = library()
        arr = (DimDesc * len(dims))(*[d.descriptor() for d in dims])
        h = ctypes.c_void_p()
        _check(lib.adsg_ctx_create(len(dims), arr, ctypes.byref(h)))
        self._h = h
        self.dims = list(dims)
        self.shape = tuple(d.dofs() for d in dims)  # (nx, ny, nz): x fastest in memory
        self.size = int(lib.adsg_ctx_size(h))

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.adsg_ctx_destroy(h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream) -> None:
        """Enqueue on a cudaStream_t (int handle, torch.cuda.Stream or None)."""
        if stream is not None and not isinstance(stream, int):
            stream = stream.cuda_stream
        _check(library().adsg_ctx_set_stream(self._h, stream))

    def synchronize(self) -> None:
        _check(library().adsg_ctx_synchronize(self._h))

    # --- stage timers -----------------------------------------------------
    def enable_stage_timers(self, on: bool = True) -> None:
        _check(library().adsg_ctx_enable_stage_timers(self._h, 1 if on else 0))

    def stage_times(self) -> dict:
        """{stage: (total_ms, launches)} accumulated since the last call (synchronises)."""
        ms = np.zeros(NSTAGES)
        n = (ctypes.c_longlong * NSTAGES)()
        _check(library().adsg_ctx_stage_times(self._h, _dptr(ms), n))
        return {STAGES[i]: (float(ms[i]), int(n[i])) for i in range(NSTAGES)}

    def solve_variants(self) -> list:
        """Line-solve variant per direction picked by the autotuner (see ads_gb300.h)."""
        v = np.zeros(3, np.int32)
        _check(library().adsg_ctx_solve_variants(self._h, _iptr(v)))
        return [int(x) for x in v[: len(self.dims)]]

    def step_solve_variants(self) -> list:
        """Line-solve variant per direction of the explicit step (see ads_gb300.h)."""
        v = np.zeros(3, np.int32)
        _check(library().adsg_ctx_step_solve_variants(self._h, _iptr(v)))
        return [int(x) for x in v[: len(self.dims)]]

    def launch_pdl(self) -> bool:
        """Whether the step's kernels use programmatic dependent launch."""
        return library().adsg_ctx_launch_pdl(self._h) == 1

    def fused_x(self) -> bool:
        """Whether heat_step fuses the x band pass into the x solve."""
        return library().adsg_ctx_fused_x(self._h) == 1

    def step_1block(self) -> bool:
        """Whether heat_step runs a whole (small 2D) step in one block."""
        return library().adsg_ctx_step_1block(self._h) == 1

    def step_cluster(self) -> bool:
        """Whether the one-launch small-grid step runs on a thread-block cluster."""
        return library().adsg_ctx_step_cluster(self._h) == 1

    def step_graphs(self) -> bool:
        """Whether heat_step replays cached single-step CUDA graphs."""
        return library().adsg_ctx_step_graphs(self._h) == 1

    def stage_work(self) -> dict:
        """{stage: (fp64_flops, hbm_bytes)} of one launch of each stage."""
        f = np.zeros(NSTAGES)
        b = np.zeros(NSTAGES)
        _check(library().adsg_ctx_stage_work(self._h, _dptr(f), _dptr(b)))
        return {STAGES[i]: (float(f[i]), float(b[i])) for i in range(NSTAGES)}

    # --- device-buffer entry points -------------------------------------
    def heat_rhs(self, u_prev, rhs, dt: float) -> None:
        _check(library().adsg_heat_rhs(self._h, _devptr(u_prev), _devptr(rhs), float(dt)))

    def heat_rhs_elem(self, u_prev, rhs, dt: float, kappa=None) -> None:
        _check(library().adsg_heat_rhs_elem(self._h, _devptr(u_prev), _devptr(kappa), _devptr(rhs), float(dt)))

    def kappa_points_count(self) -> int:
        return int(library().adsg_kappa_points_count(self._h))

    def kappa_points(self, kappa, kq) -> None:
        """kappa at every element's Gauss points (3D), for heat_rhs_elem_points."""
        _check(library().adsg_kappa_points(self._h, _devptr(kappa), _devptr(kq)))

    def heat_rhs_elem_points(self, u_prev, rhs, dt: float, kq) -> None:
        _check(library().adsg_heat_rhs_elem_points(self._h, _devptr(u_prev), _devptr(kq), _devptr(rhs), float(dt)))

    def ads_solve(self, rhs, buf=None) -> None:
        _check(library().adsg_ads_solve(self._h, _devptr(rhs), _devptr(buf)))

    def ads_solve_t(self, rhs) -> None:
        _check(library().adsg_ads_solve_t(self._h, _devptr(rhs)))

    def form_rhs(self, u, rhs, alpha: float = 0.0, beta: float = 0.0, gamma: float = 0.0, delta: float = 0.0,
                 alpha_q=None, beta_q=None, gamma_q=None, delta_q=None) -> None:
        """rhs = sum_e sum_q w J [A u v + B grad u.grad v + G v + D] with each of
        A, B, G, D a constant plus an optional Gauss-point field (device tensors
        in the layout of eval_quad); D enters without a test function."""
        f = PointForm(float(alpha), float(beta), float(gamma), float(delta), _devptr(alpha_q), _devptr(beta_q),
                      _devptr(gamma_q), _devptr(delta_q))
        _check(library().adsg_form_rhs(self._h, _devptr(u), ctypes.byref(f), _devptr(rhs)))

    def heat_step(self, u_prev, u_next, dt: float) -> None:
        """One explicit step u_next = M^-1 R u_prev (heat_3d::step)."""
        _check(library().adsg_heat_step(self._h, _devptr(u_prev), _devptr(u_next), float(dt)))

    def heat_steps(self, u, dt: float, nsteps: int) -> None:
        _check(library().adsg_heat_steps(self._h, _devptr(u), float(dt), int(nsteps)))

    def set_planes(self, u, planes) -> None:
        """Overwrite planes [(dim, index, values or None)] of a device tensor:
        the Dirichlet rows of the reference's heat_2d / validation solves."""
        arr, n = _planes(planes)
        _check(library().adsg_set_planes(self._h, _devptr(u), n, arr))

    def heat_step_dirichlet(self, u_prev, u_next, dt: float, planes) -> None:
        """heat_2d::step / validation::step: compute_rhs, the Dirichlet planes
        [(dim, index, values or None)] written into the right-hand side, then
        ads_solve with the fixed-row factorisations."""
        arr, n = _planes(planes)
        _check(library().adsg_heat_step_dirichlet(self._h, _devptr(u_prev), _devptr(u_next), float(dt), n, arr))

    def count_nonfinite(self, u) -> int:
        """Number of NaN / Inf entries of a device tensor (failure detection)."""
        c = ctypes.c_longlong()
        _check(library().adsg_count_nonfinite(self._h, _devptr(u), ctypes.byref(c)))
        return c.value

    # --- Gauss-point utilities ------------------------------------------
    @property
    def quad_size(self) -> int:
        return int(library().adsg_quad_size(self._h))

    def quad_points(self, d: int) -> np.ndarray:
        dim = self.dims[d]
        out = np.empty(dim.elements * dim.quad_order)
        _check(library().adsg_quad_points(self._h, d, _dptr(out)))
        return out

    def load_vector(self, fq, out) -> None:
        _check(library().adsg_load_vector(self._h, _devptr(fq), _devptr(out)))

    def projection(self, fq, out) -> None:
        _check(library().adsg_projection(self._h, _devptr(fq), _devptr(out)))

    def eval_quad(self, u, val, grad=None) -> None:
        _check(library().adsg_eval_quad(self._h, _devptr(u), _devptr(val), _devptr(grad)))

    def norms(self, u) -> tuple:
        l2, h1 = ctypes.c_double(), ctypes.c_double()
        _check(library().adsg_norms(self._h, _devptr(u), ctypes.byref(l2), ctypes.byref(h1)))
        return l2.value, h1.value

    def errors(self, u, fq, fgrad=None) -> tuple:
        l2, h1 = ctypes.c_double(), ctypes.c_double()
        _check(library().adsg_errors(self._h, _devptr(u), _devptr(fq), _devptr(fgrad), ctypes.byref(l2),
                                     ctypes.byref(h1)))
        return l2.value, (h1.value if h1.value >= 0 else None)

    # --- host-buffer entry points ---------------------------------------
    def heat_steps_host(self, u: np.ndarray, dt: float, nsteps: int) -> None:
        _check(library().adsg_heat_steps_host(self._h, _dptr(_host(u)), float(dt), int(nsteps)))

    def ads_solve_host(self, rhs: np.ndarray) -> None:
        _check(library().adsg_ads_solve_host(self._h, _dptr(_host(rhs))))

    def heat_rhs_host(self, u_prev: np.ndarray, rhs: np.ndarray, dt: float) -> None:
        _check(library().adsg_heat_rhs_host(self._h, _dptr(_host(u_prev)), _dptr(_host(rhs)), float(dt)))


class Heat:
    """heat_3d / heat_2d of the reference on the GPU: a state u and step(), with
    p, elements and dt as in the examples' dim_config / timesteps_config."""

    def __init__(self, ndim: int, p: int, elements: int, dt: float):
        self.dims = [Dimension(p, elements) for _ in range(ndim)]
        self.ctx = Context(self.dims)
        self.dt = dt

    def run_host(self, u: np.ndarray, steps: int) -> None:
        self.ctx.heat_steps_host(u, self.dt, steps)


class Adjoint:
    """Reverse-mode gradients of the kappa-weighted explicit heat run
    (adsg_adjoint_*): forward(u0, kappa) -> u(T) keeps sqrt(N) checkpoints;
    backward(dL/du(T)) -> (dL/du0, dL/dkappa).  Device tensors (torch)."""

    def __init__(self, ctx: Context, nsteps: int, dt: float, checkpoint_every: int = 0):
        h = ctypes.c_void_p()
        _check(library().adsg_adjoint_create(ctx.handle, int(nsteps), float(dt), int(checkpoint_every), ctypes.byref(h)))
        self._h = h
        self.ctx = ctx
        self.nsteps = nsteps
        self.dt = dt

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.adsg_adjoint_destroy(h)
            self._h = None

    def __del__(self):
        self.close()

    def checkpoints(self) -> tuple:
        e, c = ctypes.c_int(), ctypes.c_int()
        _check(library().adsg_adjoint_checkpoints(self._h, ctypes.byref(e), ctypes.byref(c)))
        return e.value, c.value

    def forward(self, u0, kappa, uT) -> None:
        _check(library().adsg_adjoint_forward(self._h, _devptr(u0), _devptr(kappa), _devptr(uT)))

    def backward(self, dL_duT, grad_u0, grad_kappa) -> None:
        _check(library().adsg_adjoint_backward(self._h, _devptr(dL_duT), _devptr(grad_u0), _devptr(grad_kappa)))


def mass_loss(ctx: Context, u, target, scratch, grad) -> float:
    """(u - target)^T M (u - target) and grad = 2 M (u - target) (adsg_mass_loss)."""
    out = ctypes.c_double()
    _check(library().adsg_mass_loss(ctx.handle, _devptr(u), _devptr(target), _devptr(scratch), ctypes.byref(out),
                                    _devptr(grad)))
    return out.value


class Batch:
    """Many independent cubic heat problems advanced by one persistent launch
    per call (adsg_batch_*).  specs: iterable of (ndim, p, elements, dt)."""

    def __init__(self, specs):
        specs = list(specs)
        self.specs = specs
        nd = np.array([s[0] for s in specs], np.int32)
        pp = np.array([s[1] for s in specs], np.int32)
        el = np.array([s[2] for s in specs], np.int32)
        dt = np.array([s[3] for s in specs], np.float64)
        h = ctypes.c_void_p()
        _check(library().adsg_batch_create(len(specs), _iptr(nd), _iptr(pp), _iptr(el), _dptr(dt), ctypes.byref(h)))
        self._h = h
        self.sizes = [int(library().adsg_batch_dofs(h, i)) for i in range(len(specs))]

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.adsg_batch_destroy(h)
            self._h = None

    def __del__(self):
        self.close()

    def set_state(self, i: int, u: np.ndarray) -> None:
        _check(library().adsg_batch_set_state(self._h, i, _dptr(_host(u))))

    def get_state(self, i: int) -> np.ndarray:
        out = np.empty(self.sizes[i])
        _check(library().adsg_batch_get_state(self._h, i, _dptr(out)))
        return out

    def steps(self, nsteps: int) -> None:
        _check(library().adsg_batch_steps(self._h, int(nsteps)))

    def steps_looped(self, nsteps: int) -> None:
        _check(library().adsg_batch_steps_looped(self._h, int(nsteps)))

    def synchronize(self) -> None:
        _check(library().adsg_batch_synchronize(self._h))

    def tuning(self) -> dict:
        b = ctypes.c_int()
        g = ctypes.c_int()
        _check(library().adsg_batch_tuning(self._h, ctypes.byref(b), ctypes.byref(g)))
        engine = library().adsg_batch_engine(self._h)
        order = library().adsg_batch_order(self._h)
        return {"blocks_per_sm": b.value, "graph": bool(g.value),
                "engine": "concurrent" if engine == 1 else "persistent",
                "order": "wavefront" if order == 1 else "stage-major"}


def batch_specs(seed: int = 0, n2d: int = 32, n3d: int = 32, dt: float = 1e-6):
    """The mixed batch: n2d 2D instances with 32..512 elements per side and n3d
    3D instances with 16..96, degrees uniform in {2, 3, 4}, drawn from a seed."""
    from .inputs import splitmix_uniform

    r = splitmix_uniform(seed, 2 * (n2d + n3d))
    specs = []
    for i in range(n2d + n3d):
        two = i < n2d
        lo, hi = (32, 512) if two else (16, 96)
        e = lo + min(int(r[2 * i] * (hi - lo + 1)), hi - lo)
        p = 2 + min(int(r[2 * i + 1] * 3), 2)
        specs.append((2 if two else 3, p, e, dt))
    return specs


def ads_solve(ctx: Context, rhs, buf=None) -> None:
    """ads::ads_solve(rhs, buf, dims...) on a device tensor; the solution is left in rhs."""
    ctx.ads_solve(rhs, buf)


def dgbtrs(trans: str, n: int, kl: int, ku: int, nrhs: int, ab: np.ndarray, ldab: int,
           ipiv: np.ndarray, b: np.ndarray, ldb: int) -> int:
    """LAPACK dgbtrs_ with the same arguments (host arrays, column-major b), solved
    on the GPU through adsg_dgbtrs_.  Returns info: 0, -k for argument k, or
    positive when b was left unsolved (a zero U diagonal at that column, or
    n + 1 when the GPU solve could not run; AdsError is raised for the latter)."""
    ab = np.ascontiguousarray(ab, dtype=np.float64)
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    _host(b)
    info = ctypes.c_int(0)
    ints = [ctypes.c_int(v) for v in (n, kl, ku, nrhs, ldab, ldb)]
    code = library().adsg_dgbtrs_(trans.encode(), ctypes.byref(ints[0]), ctypes.byref(ints[1]),
                                  ctypes.byref(ints[2]), ctypes.byref(ints[3]), _dptr(ab), ctypes.byref(ints[4]),
                                  _iptr(ipiv), _dptr(b), ctypes.byref(ints[5]), ctypes.byref(info))
    if code > 0:
        _check(code)
    return info.value


__all__ = ["AdsError", "Adjoint", "mass_loss", "Batch", "batch_specs", "Context", "DimDesc", "Dimension", "Heat", "Plane",
           "ads_solve", "debug_bounds", "dgbtrs", "library", "LIB_PATH"]
