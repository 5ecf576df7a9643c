"""filterbse_gb300 -- GB300 (sm_103a) implementation of FilterBSE's filter hot path.

The product is the C-ABI library ``libfbse_gpu.so`` (declared in
``include/fbse.h``); this module is a thin ctypes binding used by the tests,
``bench.py`` and Python callers.  Device memory is handed over as torch CUDA
tensors (torch is used only as a device allocator here).  There is no CPU
fallback: importing works without a GPU, but every compute call goes through
the CUDA library and raises if it is missing or fails.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import LIB as _LIB_PATH

__all__ = ["FbseError", "load", "Context", "samp_points", "newton_coeff", "init_filter_states",
           "FP64", "MIXED", "EXPORTED"]

FP64 = 0
MIXED = 1

EXPORTED = [
    "fbse_create", "fbse_destroy", "fbse_last_error", "fbse_version", "fbse_alloc", "fbse_free",
    "fbse_upload", "fbse_download", "fbse_sync", "fbse_stream", "fbse_hpsi", "fbse_hnorm",
    "fbse_newton_filter", "fbse_energy_range", "fbse_normalize_all", "fbse_energy_all", "fbse_sigma_e",
    "fbse_ortho_diag_sigma", "fbse_angular_stats", "fbse_samp_points", "fbse_newton_coeff", "fbse_ran",
    "fbse_init_filter_states", "fbse_launch_count", "fbse_filter_job", "fbse_build_local_pot", "fbse_build_nlc",
    "fbse_bse_potentials", "fbse_bse_kernel", "fbse_bse_kernel_real", "fbse_bse_solve", "fbse_bse_dipoles", "fbse_bse_mag_dipoles",
    "fbse_bse_qp_ang_mom",
    "fbse_bse_optical",
    "fbse_normalize_all_noalloc",
    "fbse_get_tuning", "fbse_set_tuning", "fbse_tuning_report",
    "fbse_precond_create", "fbse_precond_destroy", "fbse_precond_get_weights", "fbse_precond_set_weights",
    "fbse_precond_apply", "fbse_precond_grad", "fbse_precond_train_step", "fbse_refine",
    "fbse_gram", "fbse_rotate", "fbse_residual",
    "fbse_batch_create", "fbse_batch_run", "fbse_batch_run_sequential", "fbse_batch_graph_nodes",
    "fbse_batch_last_error", "fbse_batch_destroy",
]

PRECOND_NWEIGHTS = 15120


class FbseError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fbse error {code}: {msg}")
        self.code = code


class GridDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_long), ("ny", ctypes.c_long), ("nz", ctypes.c_long),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("ke_max", ctypes.c_double), ("nspin", ctypes.c_int), ("is_complex", ctypes.c_int),
                ("so", ctypes.c_int), ("nl", ctypes.c_int), ("dkx", ctypes.c_double), ("dky", ctypes.c_double),
                ("dkz", ctypes.c_double)]


class ProjDesc(ctypes.Structure):
    _fields_ = [("n_atoms", ctypes.c_long), ("npts", ctypes.c_long), ("nproj", ctypes.c_int),
                ("nl", ctypes.POINTER(ctypes.c_long)), ("jxyz", ctypes.POINTER(ctypes.c_int)),
                ("y1", ctypes.POINTER(ctypes.c_double)), ("so_proj", ctypes.POINTER(ctypes.c_double)),
                ("nl_proj", ctypes.POINTER(ctypes.c_double)), ("nl_sign", ctypes.POINTER(ctypes.c_int)),
                ("LS", ctypes.POINTER(ctypes.c_double))]


class BatchDot(ctypes.Structure):
    _fields_ = [("ctx", ctypes.c_void_p), ("zn", ctypes.POINTER(ctypes.c_double)),
                ("an", ctypes.POINTER(ctypes.c_double)), ("ncheby", ctypes.c_long), ("m", ctypes.c_long),
                ("vmin", ctypes.c_double), ("de", ctypes.c_double), ("psi0", ctypes.c_void_p),
                ("nstart", ctypes.c_long), ("filtered", ctypes.c_void_p)]


class Tuning(ctypes.Structure):
    """fbse_tuning: kernel choices of a context (0 = chosen by the context)."""
    _fields_ = [("fft_kernels", ctypes.c_int), ("fft_plane_cluster", ctypes.c_int),
                ("fft_chunk_blocks", ctypes.c_long), ("scatter_states", ctypes.c_int),
                ("gather_points", ctypes.c_int), ("newton_ring", ctypes.c_int), ("bse_simt", ctypes.c_int),
                ("tc_image_bytes", ctypes.c_double), ("ritz_cut", ctypes.c_double), ("ritz_hpsi", ctypes.c_int),
                ("hpsi_fused", ctypes.c_int), ("hpsi_streams", ctypes.c_int)]


_lib = None
_D = ctypes.POINTER(ctypes.c_double)
_VP = ctypes.c_void_p


def load() -> ctypes.CDLL:
    """Load libfbse_gpu.so (built in-tree by ``__graft_entry__.build()``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise FbseError(-6, f"{_LIB_PATH} is missing: build it with __graft_entry__.build()")
    L = ctypes.CDLL(_LIB_PATH)
    L.fbse_create.argtypes = [ctypes.POINTER(_VP), ctypes.POINTER(GridDesc), _D, ctypes.POINTER(ProjDesc), ctypes.c_int]
    L.fbse_destroy.argtypes = [_VP]
    L.fbse_destroy.restype = None
    L.fbse_last_error.argtypes = [_VP]
    L.fbse_last_error.restype = ctypes.c_char_p
    L.fbse_stream.argtypes = [_VP]
    L.fbse_stream.restype = _VP
    L.fbse_sync.argtypes = [_VP]
    for f in ("fbse_hpsi",):
        getattr(L, f).argtypes = [_VP, _VP, _VP, ctypes.c_long]
    L.fbse_hnorm.argtypes = [_VP, _VP, _VP, ctypes.c_long, ctypes.c_double, ctypes.c_double, ctypes.c_double]
    L.fbse_newton_filter.argtypes = [_VP, _D, _D, ctypes.c_long, ctypes.c_long, ctypes.c_double, ctypes.c_double,
                                     _VP, ctypes.c_long, _VP]
    L.fbse_energy_range.argtypes = [_VP, ctypes.c_long, ctypes.c_long, _D, _D, ctypes.POINTER(ctypes.c_long)]
    L.fbse_normalize_all.argtypes = [_VP, _VP, ctypes.c_long, _D]
    L.fbse_energy_all.argtypes = [_VP, _VP, ctypes.c_long, _D]
    L.fbse_sigma_e.argtypes = [_VP, _VP, ctypes.c_long, _D, _D]
    L.fbse_ortho_diag_sigma.argtypes = [_VP, _VP, ctypes.c_long, ctypes.POINTER(ctypes.c_long), _D, _D]
    L.fbse_samp_points.argtypes = [ctypes.c_long, _D]
    L.fbse_samp_points.restype = ctypes.c_double
    L.fbse_newton_coeff.argtypes = [ctypes.c_long, ctypes.c_long, _D, _D, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, _D]
    L.fbse_ran.argtypes = [ctypes.POINTER(ctypes.c_long)]
    L.fbse_ran.restype = ctypes.c_double
    L.fbse_init_filter_states.argtypes = [_D, ctypes.c_long, ctypes.c_long, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_long, ctypes.POINTER(ctypes.c_long)]
    L.fbse_init_filter_states.restype = ctypes.c_long
    L.fbse_launch_count.restype = ctypes.c_long
    L.fbse_launch_count.argtypes = []
    L.fbse_version.argtypes = []
    L.fbse_alloc.argtypes = [_VP, ctypes.POINTER(_VP), ctypes.c_size_t]
    L.fbse_free.argtypes = [_VP, _VP]
    L.fbse_upload.argtypes = [_VP, _VP, _VP, ctypes.c_size_t]
    L.fbse_download.argtypes = [_VP, _VP, _VP, ctypes.c_size_t]
    L.fbse_normalize_all_noalloc.argtypes = [_VP, _VP, ctypes.c_long, _VP]
    L.fbse_filter_job.argtypes = [_VP, _D, _D, ctypes.c_long, ctypes.c_long, ctypes.c_double, ctypes.c_double, _D,
                                  ctypes.c_long, ctypes.c_double, ctypes.POINTER(ctypes.c_long), _D, _D, _D]
    L.fbse_bse_potentials.argtypes = [_VP, _D, _D, _D] + [ctypes.c_double] * 6 + [_VP, _VP]
    L.fbse_bse_kernel.argtypes = [_VP, _VP, ctypes.c_long, ctypes.c_long, ctypes.c_long, _VP, _VP, _VP, _VP]
    L.fbse_bse_solve.argtypes = [_VP, _D, ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_long, _VP, _VP, _D,
                                 _VP, _D, _D, _D, _D]
    L.fbse_bse_dipoles.argtypes = [_VP, _VP, _D, _D, _D, ctypes.c_long, ctypes.c_long, ctypes.c_long, _D]
    L.fbse_bse_kernel_real.argtypes = [_VP, _VP, ctypes.c_long, ctypes.c_long, ctypes.c_long, _VP, _VP, _VP, _VP]
    L.fbse_bse_mag_dipoles.argtypes = [_VP, _VP, _D, _D, _D, ctypes.c_long, ctypes.c_long, ctypes.c_long, _D]
    L.fbse_bse_qp_ang_mom.argtypes = [_VP, _VP, _D, _D, _D, ctypes.c_long, ctypes.c_long, ctypes.c_long, _D, _D, _D,
                                      _D]
    L.fbse_bse_optical.argtypes = [_VP, _VP, _D, ctypes.c_long, ctypes.c_long, _D]
    L.fbse_angular_stats.argtypes = [_VP, _VP, ctypes.c_long, _D, _D, _D, _D]
    _Lp = ctypes.POINTER(ctypes.c_long)
    L.fbse_build_nlc.argtypes = ([ctypes.c_long] * 3 + [_D] * 3 + [ctypes.c_long, _D, _D, _D, _D, ctypes.c_int,
                                                                  ctypes.c_double, _Lp] +
                                 [ctypes.POINTER(_Lp), ctypes.POINTER(ctypes.POINTER(ctypes.c_int))] +
                                 [ctypes.POINTER(_D)] * 3)
    L.fbse_get_tuning.argtypes = [_VP, ctypes.POINTER(Tuning)]
    L.fbse_set_tuning.argtypes = [_VP, ctypes.POINTER(Tuning)]
    L.fbse_tuning_report.argtypes = [_VP, ctypes.c_char_p, ctypes.c_long]
    L.fbse_tuning_report.restype = ctypes.c_long
    L.fbse_residual.argtypes = [_VP, _VP, ctypes.c_long, _D, _VP]
    L.fbse_batch_create.argtypes = [ctypes.POINTER(_VP), ctypes.POINTER(BatchDot), ctypes.c_int]
    L.fbse_batch_run.argtypes = [_VP]
    L.fbse_batch_run_sequential.argtypes = [_VP]
    L.fbse_batch_graph_nodes.argtypes = [_VP]
    L.fbse_batch_graph_nodes.restype = ctypes.c_long
    L.fbse_batch_last_error.argtypes = [_VP]
    L.fbse_batch_last_error.restype = ctypes.c_char_p
    L.fbse_batch_destroy.argtypes = [_VP]
    L.fbse_batch_destroy.restype = None
    L.fbse_gram.argtypes = [_VP, _VP, ctypes.c_long, _VP, ctypes.c_long, ctypes.c_long, ctypes.c_long, _D]
    L.fbse_rotate.argtypes = [_VP, _VP, ctypes.c_long, _D, ctypes.c_long, ctypes.c_long, ctypes.c_long, _VP]
    _F = ctypes.POINTER(ctypes.c_float)
    L.fbse_precond_create.argtypes = [_VP, ctypes.POINTER(_VP), _F, ctypes.c_long]
    L.fbse_precond_destroy.argtypes = [_VP]
    L.fbse_precond_destroy.restype = None
    L.fbse_precond_get_weights.argtypes = [_VP, _F]
    L.fbse_precond_set_weights.argtypes = [_VP, _F]
    L.fbse_precond_apply.argtypes = [_VP, _VP, _D, ctypes.c_long, _VP]
    L.fbse_precond_grad.argtypes = [_VP, _VP, _VP, _D, ctypes.c_long, _D, _F]
    L.fbse_precond_train_step.argtypes = [_VP, _VP, _VP, _D, ctypes.c_long, ctypes.c_double, _D]
    L.fbse_refine.argtypes = [_VP, _VP, _VP, ctypes.c_long, ctypes.c_long, ctypes.c_int, ctypes.c_double,
                              ctypes.POINTER(ctypes.c_long), _D, _D]
    _lib = L
    return L


def launch_count() -> int:
    """Kernels launched by libfbse_gpu so far (all contexts)."""
    return int(load().fbse_launch_count())


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_D)


# ---------------------------------------------------------------------------
# host helpers (no GPU)
# ---------------------------------------------------------------------------

def samp_points(ncheby: int):
    zn = np.empty(ncheby)
    fk = load().fbse_samp_points(ncheby, _dp(zn))
    return zn, fk


def newton_coeff(zn, targets, vmin, de, dt):
    zn = np.ascontiguousarray(zn, np.float64)
    t = np.ascontiguousarray(targets, np.float64)
    an = np.empty(2 * len(t) * len(zn))
    rc = load().fbse_newton_coeff(len(zn), len(t), _dp(zn), _dp(t), vmin, de, dt, _dp(an))
    if rc:
        raise FbseError(rc, "fbse_newton_coeff")
    return an.view(np.complex128).reshape(len(t), len(zn))


def init_filter_states(n_filters, ngrid, nspin, is_complex, dv, seed):
    stlen = (2 if is_complex else 1) * nspin * ngrid
    out = np.empty(n_filters * stlen)
    seeds = np.empty(n_filters * nspin, np.int64)
    s = load().fbse_init_filter_states(_dp(out), n_filters, ngrid, nspin, int(is_complex), dv, seed,
                                       seeds.ctypes.data_as(ctypes.POINTER(ctypes.c_long)))
    return out.reshape(n_filters, stlen), seeds, s


def build_nlc(axes, xyz, so_par, so_tab, nl_tab, nproj, rcut2):
    """init_NL_projectors on the GPU (fbse_build_nlc): the projector table of
    the atoms xyz [nat, 3] on the grid with coordinates axes = (gx, gy, gz).
    so_tab [nproj, 1024] (scaled per atom by sqrt(so_par)) and nl_tab
    [nat, nproj, 1024] may be None.  Returns (nl, npts, jxyz, y1, so_p, nl_p)
    as numpy arrays (row stride npts)."""
    L = load()
    gx, gy, gz = (np.ascontiguousarray(a, np.float64) for a in axes)
    xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
    nat = len(xyz)
    sp = None if so_par is None else np.ascontiguousarray(so_par, np.float64)
    st = None if so_tab is None else np.ascontiguousarray(so_tab, np.float64)
    nt = None if nl_tab is None else np.ascontiguousarray(nl_tab, np.float64)
    opt = lambda a: _dp(a) if a is not None else None
    npts = ctypes.c_long()
    p_nl = ctypes.POINTER(ctypes.c_long)()
    p_jx = ctypes.POINTER(ctypes.c_int)()
    p_y1, p_so, p_np = _D(), _D(), _D()
    rc = L.fbse_build_nlc(len(gx), len(gy), len(gz), _dp(gx), _dp(gy), _dp(gz), nat, _dp(xyz), opt(sp), opt(st),
                          opt(nt), int(nproj), float(rcut2), ctypes.byref(npts), ctypes.byref(p_nl),
                          ctypes.byref(p_jx), ctypes.byref(p_y1), ctypes.byref(p_so), ctypes.byref(p_np))
    if rc:
        raise FbseError(rc, "fbse_build_nlc")
    n = max(nat, 1) * npts.value
    out = (np.ctypeslib.as_array(p_nl, (max(nat, 1),))[:nat].copy(), npts.value,
           np.ctypeslib.as_array(p_jx, (n,)).copy(), np.ctypeslib.as_array(p_y1, (n * 6,)).copy(),
           np.ctypeslib.as_array(p_so, (n * nproj,)).copy(), np.ctypeslib.as_array(p_np, (n * nproj,)).copy())
    libc = ctypes.CDLL(None)
    libc.free.argtypes = [ctypes.c_void_p]
    for p in (p_nl, p_jx, p_y1, p_so, p_np):
        libc.free(ctypes.cast(p, ctypes.c_void_p))
    return out


# ---------------------------------------------------------------------------
# device context
# ---------------------------------------------------------------------------

class Context:
    """One fbse_ctx: grid, local potential, projector table, FFT plans.

    grid: object/dict with nx, ny, nz, dx, dy, dz, ke_max; nspin, is_complex,
    so, nl switches.  proj: object with nl, npts, jxyz, y1, proj (SO radial),
    nlp (NL radial), sgn, nproj (the layout of the reference's nlc_st array)."""

    def __init__(self, grid, pot, *, nspin=1, is_complex=False, so=False, nl=False, proj=None,
                 precision=FP64, LS=None):
        L = load()
        dk = grid.dk() if hasattr(grid, "dk") else (0.0, 0.0, 0.0)
        g = GridDesc(int(grid.nx), int(grid.ny), int(grid.nz), float(grid.dx), float(grid.dy), float(grid.dz),
                     float(grid.ke_max), int(nspin), int(bool(is_complex)), int(bool(so)), int(bool(nl)),
                     float(dk[0]), float(dk[1]), float(dk[2]))
        self._keep = []
        pd = None
        if proj is not None and (so or nl):
            nlc = np.ascontiguousarray(proj.nl, np.int64)
            jx = np.ascontiguousarray(proj.jxyz, np.int32)
            y1 = np.ascontiguousarray(proj.y1, np.float64)
            sp = np.ascontiguousarray(proj.proj, np.float64)
            npj = np.ascontiguousarray(proj.nlp, np.float64)
            sg = np.ascontiguousarray(proj.sgn, np.int32)
            ls = None if LS is None else np.ascontiguousarray(np.asarray(LS, np.complex128)).view(np.float64)
            self._keep += [nlc, jx, y1, sp, npj, sg, ls]
            pd = ProjDesc(len(nlc), int(proj.npts), int(proj.nproj), nlc.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                          jx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(y1), _dp(sp), _dp(npj),
                          sg.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(ls) if ls is not None else None)
        pot = np.ascontiguousarray(pot, np.float64)
        h = _VP()
        rc = L.fbse_create(ctypes.byref(h), ctypes.byref(g), _dp(pot), ctypes.byref(pd) if pd else None, precision)
        self._h = h
        self._L = L
        if rc:
            msg = L.fbse_last_error(h).decode() if h.value else "no CUDA device"
            self.close()
            raise FbseError(rc, msg)
        self.grid = grid
        self.nspin = nspin
        self.is_complex = bool(is_complex)
        self.precision = precision
        self.ngrid = int(grid.nx) * int(grid.ny) * int(grid.nz)
        self.stlen = (2 if is_complex else 1) * nspin * self.ngrid

    # -- plumbing -------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.fbse_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        if rc:
            raise FbseError(rc, self._L.fbse_last_error(self._h).decode())

    @property
    def stream_handle(self) -> int:
        return int(self._L.fbse_stream(self._h) or 0)

    def sync(self):
        self._chk(self._L.fbse_sync(self._h))

    # -- kernel choices -----------------------------------------------------------
    def get_tuning(self) -> dict:
        t = Tuning()
        self._chk(self._L.fbse_get_tuning(self._h, ctypes.byref(t)))
        return {f: getattr(t, f) for f, _ in Tuning._fields_}

    def set_tuning(self, **fields):
        """Fix kernel choices (fbse_tuning fields; 0 = chosen by the context)."""
        cur = self.get_tuning()
        for k, v in fields.items():
            if k not in cur:
                raise KeyError(k)
            cur[k] = v
        self._chk(self._L.fbse_set_tuning(self._h, ctypes.byref(Tuning(**cur))))

    def tuning_report(self) -> list:
        import json
        n = self._L.fbse_tuning_report(self._h, None, 0)
        buf = ctypes.create_string_buffer(n + 1)
        self._L.fbse_tuning_report(self._h, buf, n + 1)
        return json.loads(buf.value.decode())

    @staticmethod
    def _ptr(t):
        import torch
        assert t.is_cuda and t.is_contiguous()
        return ctypes.c_void_p(t.data_ptr())

    @staticmethod
    def _torch_sync():
        import torch
        torch.cuda.current_stream().synchronize()

    def working_dtype(self):
        import torch
        return torch.complex64 if self.precision == MIXED else torch.complex128

    # -- operators --------------------------------------------------------------
    def hpsi(self, psi_in, psi_out, sync=True):
        """psi_out = H psi_in for [n, nspin*ngrid] complex tensors (working precision)."""
        self._torch_sync()
        n = psi_in.shape[0] if psi_in.dim() > 1 else 1
        self._chk(self._L.fbse_hpsi(self._h, self._ptr(psi_in), self._ptr(psi_out), n))
        if sync:
            self.sync()

    def hnorm(self, psi_in, psi_out, vmin, de, zn, sync=True):
        self._torch_sync()
        n = psi_in.shape[0] if psi_in.dim() > 1 else 1
        self._chk(self._L.fbse_hnorm(self._h, self._ptr(psi_in), self._ptr(psi_out), n, vmin, de, zn))
        if sync:
            self.sync()

    def newton_filter(self, zn, an, vmin, de, psi0, out=None):
        """filter_cycle for all starts: psi0 [nstart, stlen] float64 CUDA tensor;
        returns [nstart, m, stlen] float64 CUDA tensor (psi_rank layout)."""
        import torch
        zn = np.ascontiguousarray(zn, np.float64)
        an = np.ascontiguousarray(an, np.complex128)
        m, nc = an.shape
        nstart = psi0.shape[0]
        if out is None:
            out = torch.empty((nstart, m, self.stlen), dtype=torch.float64, device=psi0.device)
        anv = an.view(np.float64).reshape(-1)
        self._torch_sync()
        self._chk(self._L.fbse_newton_filter(self._h, _dp(zn), _dp(anv), nc, m, vmin, de, self._ptr(psi0), nstart,
                                             self._ptr(out)))
        return out

    def energy_range(self, seed=-874917403, max_iter=1500):
        e0 = ctypes.c_double()
        e1 = ctypes.c_double()
        it = ctypes.c_long()
        self._chk(self._L.fbse_energy_range(self._h, seed, max_iter, ctypes.byref(e0), ctypes.byref(e1),
                                            ctypes.byref(it)))
        return e0.value, e1.value, it.value

    def normalize_all(self, psitot):
        n = psitot.shape[0]
        norms = np.empty(n)
        self._torch_sync()
        self._chk(self._L.fbse_normalize_all(self._h, self._ptr(psitot), n, _dp(norms)))
        return norms

    def energy_all(self, psitot):
        n = psitot.shape[0]
        e = np.empty(n)
        self._torch_sync()
        self._chk(self._L.fbse_energy_all(self._h, self._ptr(psitot), n, _dp(e)))
        return e

    def sigma_e(self, psitot):
        """calc_sigma_E: (eval, sigma) of n psitot states (device)."""
        n = psitot.shape[0]
        e = np.empty(n)
        sg = np.empty(n)
        self._torch_sync()
        self._chk(self._L.fbse_sigma_e(self._h, self._ptr(psitot), n, _dp(e), _dp(sg)))
        return e, sg

    def filter_job(self, zn, an, vmin, de, psi0_host, sigma_cut=0.0, psi_out=None):
        """Whole filter stage on host buffers (fbse_filter_job): returns
        (n, eval, sigma); psi_out (host float64 [nstart*m, stlen], optional,
        ideally pinned) receives the returned states."""
        zn = np.ascontiguousarray(zn, np.float64)
        an = np.ascontiguousarray(an, np.complex128)
        m, nc = an.shape
        p0 = np.ascontiguousarray(psi0_host, np.float64)
        nstart = p0.shape[0]
        ev = np.empty(nstart * m)
        sg = np.empty(nstart * m)
        nout = ctypes.c_long()
        pp = None
        if psi_out is not None:
            pp = ctypes.cast(ctypes.c_void_p(psi_out.data_ptr() if hasattr(psi_out, "data_ptr")
                                             else psi_out.ctypes.data), _D)
        self._chk(self._L.fbse_filter_job(self._h, _dp(zn), _dp(an.view(np.float64).reshape(-1)), nc, m, vmin, de,
                                          _dp(p0), nstart, sigma_cut, ctypes.byref(nout), _dp(ev), _dp(sg), pp))
        k = nout.value
        return k, ev[:k].copy(), sg[:k].copy()

    def ortho_diag_sigma(self, psitot):
        n = psitot.shape[0]
        ev = np.empty(n)
        sg = np.empty(n)
        nk = ctypes.c_long()
        self._torch_sync()
        self._chk(self._L.fbse_ortho_diag_sigma(self._h, self._ptr(psitot), n, ctypes.byref(nk), _dp(ev), _dp(sg)))
        k = nk.value
        return k, ev[:k].copy(), sg[:k].copy()

    def gram(self, A, B, off=0, length=None):
        """dv-weighted overlap conj(A) B^T over a slab of points (fbse_gram):
        A [na, stlen], B [nb, stlen] device float64; returns complex128 [na, nb]."""
        L = self.nspin * self.ngrid
        length = L - off if length is None else length
        out = np.empty((A.shape[0], B.shape[0]), np.complex128)
        self._torch_sync()
        self._chk(self._L.fbse_gram(self._h, self._ptr(A), A.shape[0], self._ptr(B), B.shape[0], off, length,
                                    out.view(np.float64).ctypes.data_as(_D)))
        return out

    def rotate(self, A, coef, out, off=0, length=None):
        """out_j = sum_i coef[i, j] A_i over a slab (fbse_rotate); coef
        complex [na, k] host, out device float64 [>= k, stlen]."""
        L = self.nspin * self.ngrid
        length = L - off if length is None else length
        cf = np.ascontiguousarray(coef, np.complex128)
        self._torch_sync()
        self._chk(self._L.fbse_rotate(self._h, self._ptr(A), A.shape[0], cf.view(np.float64).ctypes.data_as(_D),
                                      cf.shape[1], off, length, self._ptr(out)))
        return out

    def residual(self, psitot, ene):
        """H psi_i - ene_i psi_i of psitot rows (fbse_residual); device float64."""
        import torch
        out = torch.empty_like(psitot)
        e = np.ascontiguousarray(ene, np.float64)
        self._torch_sync()
        self._chk(self._L.fbse_residual(self._h, self._ptr(psitot), psitot.shape[0], _dp(e), self._ptr(out)))
        return out

    def refine(self, psitot, n, ev, sg, steps=2, tol=1e-2, precond=None):
        """fbse_refine: residual refinement of the first n Ritz pairs of
        psitot [cap, stlen] (device float64, normalised Ritz vectors, with
        their eval / sigma); returns (n_out, eval, sigma)."""
        cap = psitot.shape[0]
        e = np.zeros(cap)
        s_ = np.zeros(cap)
        e[:n] = ev[:n]
        s_[:n] = sg[:n]
        nk = ctypes.c_long()
        self._torch_sync()
        self._chk(self._L.fbse_refine(self._h, precond._p if precond is not None else None, self._ptr(psitot), n, cap,
                                      steps, tol, ctypes.byref(nk), _dp(e), _dp(s_)))
        k = nk.value
        return k, e[:k].copy(), s_[:k].copy()

    # -- Bethe-Salpeter stage -----------------------------------------------------
    def bse_potentials(self, gx, gy, gz, xmin, ymin, zmin, eps=(6.0, 6.0, 6.0)):
        """init_elec_hole_kernel: returns (pot_bare, pot_screened), [ngrid]
        complex128 CUDA tensors."""
        import torch
        gx, gy, gz = (np.ascontiguousarray(a, np.float64) for a in (gx, gy, gz))
        bare = torch.empty(self.ngrid, dtype=torch.complex128, device="cuda")
        scr = torch.empty_like(bare)
        self._torch_sync()
        self._chk(self._L.fbse_bse_potentials(self._h, _dp(gx), _dp(gy), _dp(gz), xmin, ymin, zmin, eps[0], eps[1],
                                              eps[2], self._ptr(bare), self._ptr(scr)))
        return bare, scr

    def bse_kernel(self, psi_qp, n_h, n_e, lumo_idx, pot_bare, pot_screened):
        """calc_eh_kernel_cplx: psi_qp [n_qp, nspin*ngrid] complex128 CUDA;
        returns (direct, exchange) [n_xton, n_xton] complex128, lower triangles."""
        import torch
        n = n_h * n_e
        d = torch.zeros((n, n), dtype=torch.complex128, device=psi_qp.device)
        x = torch.zeros_like(d)
        self._torch_sync()
        self._chk(self._L.fbse_bse_kernel(self._h, self._ptr(psi_qp), n_h, n_e, lumo_idx, self._ptr(pot_bare),
                                          self._ptr(pot_screened), self._ptr(d), self._ptr(x)))
        return d, x

    def bse_kernel_real(self, psi_qp, n_h, n_e, lumo_idx, pot_bare, pot_screened):
        """calc_eh_kernel_cplx of bse_real: psi_qp [n_qp, ngrid] float64 CUDA
        (real states, nspin = 1); returns (direct, exchange) [n_xton, n_xton]
        float64, lower triangles, exchange with the singlet factor 2."""
        import torch
        n = n_h * n_e
        d = torch.zeros((n, n), dtype=torch.float64, device=psi_qp.device)
        x = torch.zeros_like(d)
        self._torch_sync()
        self._chk(self._L.fbse_bse_kernel_real(self._h, self._ptr(psi_qp), n_h, n_e, lumo_idx, self._ptr(pot_bare),
                                               self._ptr(pot_screened), self._ptr(d), self._ptr(x)))
        return d, x

    def bse_solve(self, eval_qp, n_h, n_e, lumo_idx, direct, exchange):
        """build_BSE_mat + bethe_salpeter: returns (xton_ene, coeff, <H>, <Kd>,
        <Kx>, <h0>); coeff [n_xton, n_xton] complex128 CUDA, column j = exciton j.
        direct/exchange are completed to Hermitian matrices in place."""
        import torch
        ev = np.ascontiguousarray(eval_qp, np.float64)
        n = n_h * n_e
        coeff = torch.empty((n, n), dtype=torch.complex128, device=direct.device)
        e, h, dd, xx, h0 = (np.empty(n) for _ in range(5))
        self._torch_sync()
        self._chk(self._L.fbse_bse_solve(self._h, _dp(ev), len(ev), n_h, n_e, lumo_idx, self._ptr(direct),
                                         self._ptr(exchange), _dp(e), self._ptr(coeff), _dp(h), _dp(dd), _dp(xx),
                                         _dp(h0)))
        return e, coeff, h, dd, xx, h0

    def bse_dipoles(self, psi_qp, gx, gy, gz, n_h, n_e, lumo_idx):
        """calc_elec_dipole: returns mu [n_h*n_e, 3] complex128 (numpy), row i*n_e+a."""
        gx, gy, gz = (np.ascontiguousarray(a, np.float64) for a in (gx, gy, gz))
        mu = np.empty(n_h * n_e * 3, np.complex128)
        self._torch_sync()
        self._chk(self._L.fbse_bse_dipoles(self._h, self._ptr(psi_qp), _dp(gx), _dp(gy), _dp(gz), n_h, n_e,
                                           lumo_idx, _dp(mu.view(np.float64))))
        return mu.reshape(-1, 3)

    def bse_mag_dipoles(self, psi_qp, gx, gy, gz, n_h, n_e, lumo_idx):
        """calc_mag_dipole: returns m [n_h*n_e, 3] complex128 (numpy), row i*n_e+a."""
        gx, gy, gz = (np.ascontiguousarray(a, np.float64) for a in (gx, gy, gz))
        m = np.empty(n_h * n_e * 3, np.complex128)
        self._torch_sync()
        self._chk(self._L.fbse_bse_mag_dipoles(self._h, self._ptr(psi_qp), _dp(gx), _dp(gy), _dp(gz), n_h, n_e,
                                               lumo_idx, _dp(m.view(np.float64))))
        return m.reshape(-1, 3)

    def bse_qp_ang_mom(self, psi_qp, gx, gy, gz, n_h, n_e, lumo_idx):
        """calc_qp_spin_mtrx + calc_qp_ang_mom_mtrx: (s [n,3], l [n,3], l2 [n],
        ls [n]) complex128 with n = n_h^2 + n_e^2 (holes first)."""
        gx, gy, gz = (np.ascontiguousarray(a, np.float64) for a in (gx, gy, gz))
        n = n_h * n_h + n_e * n_e
        s = np.empty(n * 3, np.complex128)
        l = np.empty(n * 3, np.complex128)
        l2 = np.empty(n, np.complex128)
        ls = np.empty(n, np.complex128)
        self._torch_sync()
        self._chk(self._L.fbse_bse_qp_ang_mom(self._h, self._ptr(psi_qp), _dp(gx), _dp(gy), _dp(gz), n_h, n_e,
                                              lumo_idx, _dp(s.view(np.float64)), _dp(l.view(np.float64)),
                                              _dp(l2.view(np.float64)), _dp(ls.view(np.float64))))
        return s.reshape(-1, 3), l.reshape(-1, 3), l2, ls

    def angular_stats(self, states, gx, gy, gz):
        """calc_angular_exp (filter_mpi/angular.c:4-165): per complex spinor
        state (device, psitot layout), the angular.dat columns <Jx>, <Jx^2>,
        <Jy>, <Jy^2>, <Jz>, <Jz^2>, <J^2>, norm as an [n, 8] array."""
        gx, gy, gz = (np.ascontiguousarray(a, np.float64) for a in (gx, gy, gz))
        n = int(states.shape[0])
        out = np.empty((n, 8), np.float64)
        self._torch_sync()
        self._chk(self._L.fbse_angular_stats(self._h, self._ptr(states), n, _dp(gx), _dp(gy), _dp(gz), _dp(out)))
        return out

    def bse_optical(self, coeff, mu_pairs, n_h, n_e):
        """calc_optical_exc (electric part): exciton dipoles [n_xton, 3] complex128
        and the oscillator-strength columns of OS.dat given xton energies later."""
        mp = np.ascontiguousarray(mu_pairs, np.complex128)
        out = np.empty(n_h * n_e * 3, np.complex128)
        self._torch_sync()
        self._chk(self._L.fbse_bse_optical(self._h, self._ptr(coeff), _dp(mp.reshape(-1).view(np.float64)), n_h, n_e,
                                           _dp(out.view(np.float64))))
        return out.reshape(-1, 3)


class Precond:
    """The learned residual preconditioner of a context (fbse_precond_*):
    4 convolutions 3x3x3, 16 channels, FP32 weights, BF16 activations."""

    def __init__(self, ctx: Context, weights=None, seed: int = 1):
        self.ctx = ctx
        self._L = ctx._L
        self._p = ctypes.c_void_p()
        w = None
        if weights is not None:
            w = np.ascontiguousarray(weights, np.float32)
            assert w.size == PRECOND_NWEIGHTS
        rc = self._L.fbse_precond_create(ctx._h, ctypes.byref(self._p),
                                         w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if w is not None else None,
                                         seed)
        ctx._chk(rc)

    def close(self):
        if self._p:
            self._L.fbse_precond_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def weights(self) -> np.ndarray:
        w = np.empty(PRECOND_NWEIGHTS, np.float32)
        self.ctx._chk(self._L.fbse_precond_get_weights(self._p, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return w

    @weights.setter
    def weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        assert w.size == PRECOND_NWEIGHTS
        self.ctx._chk(self._L.fbse_precond_set_weights(self._p, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def apply(self, resid, ene):
        """P(resid) for resid [n, stlen] (device float64 psitot), ene [n]."""
        import torch
        out = torch.empty_like(resid)
        e = np.ascontiguousarray(ene, np.float64)
        self.ctx._torch_sync()
        self.ctx._chk(self._L.fbse_precond_apply(self._p, self.ctx._ptr(resid), _dp(e), resid.shape[0],
                                                 self.ctx._ptr(out)))
        return out

    def grad(self, resid, corr, ene):
        """(loss, gradient [PRECOND_NWEIGHTS] float32) without a step."""
        e = np.ascontiguousarray(ene, np.float64)
        g = np.empty(PRECOND_NWEIGHTS, np.float32)
        loss = ctypes.c_double()
        self.ctx._torch_sync()
        self.ctx._chk(self._L.fbse_precond_grad(self._p, self.ctx._ptr(resid), self.ctx._ptr(corr), _dp(e),
                                                resid.shape[0], ctypes.byref(loss),
                                                g.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return loss.value, g

    def train_step(self, resid, corr, ene, lr=1e-3) -> float:
        e = np.ascontiguousarray(ene, np.float64)
        loss = ctypes.c_double()
        self.ctx._torch_sync()
        self.ctx._chk(self._L.fbse_precond_train_step(self._p, self.ctx._ptr(resid), self.ctx._ptr(corr), _dp(e),
                                                      resid.shape[0], lr, ctypes.byref(loss)))
        return loss.value


class Batch:
    """Multi-dot filter in one CUDA graph (fbse_batch_*).  dots: list of
    (ctx, zn, an, vmin, de, psi0 device [nstart, stlen]); filtered outputs are
    allocated here ([nstart, m, stlen] float64 CUDA tensors, ``self.out``)."""

    def __init__(self, dots):
        import torch
        self._L = load()
        self._keep = []
        arr = (BatchDot * len(dots))()
        self.out = []
        for i, (ctx, zn, an, vmin, de, psi0) in enumerate(dots):
            zn = np.ascontiguousarray(zn, np.float64)
            an = np.ascontiguousarray(an, np.complex128)
            m, nc = an.shape
            anv = an.view(np.float64).reshape(-1)
            out = torch.empty((psi0.shape[0], m, ctx.stlen), dtype=torch.float64, device=psi0.device)
            self._keep += [zn, anv, psi0, out]
            self.out.append(out)
            arr[i] = BatchDot(ctx._h, _dp(zn), _dp(anv), nc, m, vmin, de, psi0.data_ptr(), psi0.shape[0],
                              out.data_ptr())
        torch.cuda.current_stream().synchronize()
        self._b = ctypes.c_void_p()
        rc = self._L.fbse_batch_create(ctypes.byref(self._b), arr, len(dots))
        if rc:
            msg = self._L.fbse_batch_last_error(self._b).decode() if self._b else ""
            if self._b:
                self._L.fbse_batch_destroy(self._b)
                self._b = ctypes.c_void_p()
            raise FbseError(rc, msg)

    @property
    def nodes(self) -> int:
        return int(self._L.fbse_batch_graph_nodes(self._b))

    def run(self, sequential=False):
        f = self._L.fbse_batch_run_sequential if sequential else self._L.fbse_batch_run
        rc = f(self._b)
        if rc:
            raise FbseError(rc, self._L.fbse_batch_last_error(self._b).decode())

    def close(self):
        if self._b:
            self._L.fbse_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
