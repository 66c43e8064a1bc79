"""Python binding of libtg3.so (the GB300 E-step + insertion library).

This is plumbing over the C ABI declared in include/thunder_gb300.h: ctypes
signatures, status checking, and helpers that pass torch CUDA tensors (device
pointers) or numpy arrays (host pointers).  There is no compute here and no
fallback: if the shared library is missing the import of `lib()` fails.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parents[1]
LIB_PATH = PKG / "libtg3.so"

OK, ERR_ARG, ERR_CUDA, ERR_ALLOC, ERR_STATE, ERR_TIMEOUT, ERR_NUMERIC, ERR_UNSUPPORTED = range(8)
KERNEL_TRILINEAR, KERNEL_MKB = 0, 1
SCORE_FP32, SCORE_BF16X3 = 0, 1

# every extern "C" symbol declared in include/thunder_gb300.h
EXPORTS = [
    "tg3_status_string", "tg3_last_error", "tg3_version", "tg3_getAviDevice",
    "tg3_ExpectRotran", "tg3_ExpectProject", "tg3_ExpectGlobal3D", "tg3_InsertFT",
    "tg3_volume_create", "tg3_volume_destroy", "tg3_ExpectLocal3D", "tg3_resample",
    "tg3_ctx_create", "tg3_ctx_destroy", "tg3_ctx_stream", "tg3_ctx_sync",
    "tg3_ctx_workspace_bytes", "tg3_ctx_set_volume", "tg3_ctx_set_pixels",
    "tg3_local_phase_d", "tg3_resample_d", "tg3_ctx_insert_begin", "tg3_insert_d",
    "tg3_ctx_insert_read_d", "tg3_ctx_insert_ratio_d", "tg3_fsc_d", "tg3_rotmat_d", "tg3_translate_d", "tg3_ctf_d",
    "tg3_project_d", "tg3_ctx_render_references_d", "tg3_local_phase", "tg3_ctx_set_timing", "tg3_ctx_stage_times",
    "tg3_ctx_set_option", "tg3_ctx_set_pixels_slot", "tg3_ctx_use_pixels",
    "tg3_ragged_plan_create", "tg3_ragged_plan_run", "tg3_ragged_plan_info",
    "tg3_ragged_plan_kblock", "tg3_ragged_plan_project_group", "tg3_Reconstruct2D", "tg3_SymmetrizeO",
    "tg3_ragged_plan_destroy", "tg3_cnn_create", "tg3_cnn_destroy", "tg3_cnn_param_count",
    "tg3_cnn_params", "tg3_cnn_grads", "tg3_cnn_set_bf16", "tg3_cnn_forward", "tg3_cnn_loss",
    "tg3_cnn_zero_grads", "tg3_cnn_adam", "tg3_cnn_propose", "tg3_cnn_backward", "tg3_cnn_infer",
    "tg3_cnn_contrastive", "tg3_cnn_embed", "tg3_cnn_match_propose", "tg3_ctx_set_bank",
    "tg3_local_phase_bank_d", "tg3_local_phase_ctf_d", "tg3_ExpectLocal3D_ctf",
    "tg3_ExpectGlobal2D", "tg3_global_scan2d_d", "tg3_InsertI2D", "tg3_global_scan2d_classes_d",
    "tg3_prepare_images_d", "tg3_sigma_d", "tg3_ctx_reconstruct_d", "tg3_ctx_insert_load_d",
    "tg3_mrc_info", "tg3_mrc_read", "tg3_mrc_write", "tg3_thu_count",
    "tg3_thu_read", "tg3_thu_write",
    "tg3_noalloc_scratch_bytes", "tg3_local_phase_noalloc", "tg3_global_scan_d",
    "tg3_ctx_set_references", "tg3_learned_expect_d", "tg3_ExpectLearned3D",
    "tg3_InsertFT_classes", "tg3_remask_d", "tg3_ReMask", "tg3_ctx_prepare_tf_d",
    "tg3_PrepareTF", "tg3_image_create", "tg3_image_destroy", "tg3_ExpectLocal2D",
]
STAGES = ("project", "shift", "cross", "weights", "resample", "insert", "fused", "network",
          "fallback", "fallback_cross", "norm")
OPT_FUSED = 0
OPT_INSERT_GATHER = 1
OPT_BANK_GATHER = 2
OPT_BANK_ORDER = 3
OPT_SCAN_TILE_N = 4
OPT_SCAN_PAIR = 5
OPT_SCAN_BK = 6
OPT_LOCAL_BK = 7
OPT_PROJECT_FORM = 8
OPT_BANK_SHAPE = 9
OPT_PROJECT_GROUP = 10


class TG3Error(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"tg3 status {status}: {msg}")
        self.status = status


class LearnedOut(ctypes.Structure):
    """tg3_learned_out: device pointers of the learned E-step's outputs."""
    _fields_ = [(k, ctypes.c_void_p) for k in (
        "bestQuat", "bestTrans", "baseL", "peak", "fellBack", "propIdx", "propQuat",
        "propTrans", "propWR", "propWT", "propBase", "propDvp")]


_lib = None
_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_F = ctypes.c_float


def lib():
    """Load libtg3.so (built by tg3.build / __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: build the CUDA library first "
                              "(python -c 'import __graft_entry__ as g; g.build()')")
        L = ctypes.CDLL(str(LIB_PATH))
        sig = {
            "tg3_status_string": ([_I], ctypes.c_char_p),
            "tg3_last_error": ([], ctypes.c_char_p),
            "tg3_version": ([], ctypes.c_char_p),
            "tg3_getAviDevice": ([_P, _I, _P], _I),
            "tg3_ExpectRotran": ([_P, _P, _P, _P, _P, _P, _I, _I, _I, _I], _I),
            "tg3_ExpectProject": ([_P, _P, _P, _P, _P, _I, _I, _I, _I, _I], _I),
            "tg3_ExpectGlobal3D": ([_P] * 11 + [_I] * 6, _I),
            "tg3_InsertFT": ([_P] * 15 + [_F, _I, _I, _I, _I, _I, _I, _I, _I], _I),
            "tg3_InsertFT_classes": ([_P] * 16 + [_F, _I, _I, _I, _I, _I, _I, _I, _I], _I),
            "tg3_remask_d": ([_P, _P, _I, _I, _F, _F, _P], _I),
            "tg3_ReMask": ([_P, _I, _I, _F, _F, _F], _I),
            "tg3_ctx_prepare_tf_d": ([_P, _P, _I, _I, _I], _I),
            "tg3_PrepareTF": ([_P, _P, _I, _P, _I, _I, _I], _I),
            "tg3_image_create": ([_P, _P, _I, _I], _I),
            "tg3_image_destroy": ([_P], _I),
            "tg3_ExpectLocal2D": ([_P, _P, _P, _P, _P, _P, _I, _I, _P, _I, _P, _I, _P, _P, _D,
                                   _P, _P, _P, _P, _P], _I),
            "tg3_volume_create": ([_P, _P, _I, _I], _I),
            "tg3_volume_destroy": ([_P], _I),
            "tg3_ExpectLocal3D": ([_P, _P, _P, _P, _P, _P, _I, _I, _P, _I, _P, _I, _P, _P, _D,
                                   _P, _P, _P, _P, _P], _I),
            "tg3_resample": ([_I, _I, _P, _P, _P, _P, _P, _I, _P, _P, _P], _I),
            "tg3_ctx_create": ([_P, _I], _I),
            "tg3_ctx_destroy": ([_P], _I),
            "tg3_ctx_stream": ([_P], _P),
            "tg3_ctx_sync": ([_P], _I),
            "tg3_ctx_workspace_bytes": ([_P], ctypes.c_size_t),
            "tg3_ctx_set_volume": ([_P, _I, _P, _I, _I, _I], _I),
            "tg3_ctx_set_pixels": ([_P, _P, _P, _I, _I], _I),
            "tg3_local_phase_d": ([_P, _I, _I, _I] + [_P] * 14 + [_I], _I),
            "tg3_resample_d": ([_P, _I, _I, _P, _P, _P, _P, _P, _I, _P, _P, _P], _I),
            "tg3_ctx_insert_begin": ([_P, _I, _I], _I),
            "tg3_insert_d": ([_P, _I, _P, _P, _P, _P, _P, _P, _I, _P, _P], _I),
            "tg3_ctx_insert_read_d": ([_P, _P, _P, _I], _I),
            "tg3_ctx_insert_ratio_d": ([_P, _P, _F], _I),
            "tg3_fsc_d": ([_P, _P, _I, _I, _P, _P, _P], _I),
            "tg3_rotmat_d": ([_P, _I, _P, _P], _I),
            "tg3_translate_d": ([_P, _I, _I, _P, _P, _I, _P, _P], _I),
            "tg3_ctf_d": ([_P, _I, _F, _I, _P, _P, _I, _P, _P], _I),
            "tg3_project_d": ([_P, _I, _P, _I, _P], _I),
            "tg3_ctx_render_references_d": ([_P, _I, _P, _I, _I, _P], _I),
            "tg3_local_phase": ([_P, _I, _I, _I] + [_P] * 14 + [_I], _I),
            "tg3_ctx_set_timing": ([_P, _I], _I),
            "tg3_ctx_set_option": ([_P, _I, _I], _I),
            "tg3_ctx_set_pixels_slot": ([_P, _I, _P, _P, _I, _I], _I),
            "tg3_ctx_use_pixels": ([_P, _I], _I),
            "tg3_ragged_plan_create": ([_P, _I] + [_P] * 27 + [_I, ctypes.c_size_t, _I, _P], _I),
            "tg3_ragged_plan_run": ([_P], _I),
            "tg3_ragged_plan_info": ([_P, _P, _P], _I),
            "tg3_ragged_plan_kblock": ([_P, _P], _I),
            "tg3_ragged_plan_project_group": ([_P, _P], _I),
            "tg3_Reconstruct2D": ([_P, _P, _I, _I, _P, _I, _I, _I, _I, _I, ctypes.c_float,
                                   ctypes.c_float, _P, _P], _I),
            "tg3_SymmetrizeO": ([_P, _P, _P, _I], _I),
            "tg3_ragged_plan_destroy": ([_P], _I),
            "tg3_cnn_create": ([_P, _I, ctypes.c_ulonglong], _I),
            "tg3_cnn_destroy": ([_P], _I),
            "tg3_cnn_param_count": ([_P], ctypes.c_size_t),
            "tg3_cnn_params": ([_P, _P, _I], _I),
            "tg3_cnn_grads": ([_P, _P], _I),
            "tg3_cnn_set_bf16": ([_P, _I], _I),
            "tg3_cnn_forward": ([_P, _P, _I, _P], _I),
            "tg3_cnn_loss": ([_P, _P, _I, _P, _P, _I, _P], _I),
            "tg3_cnn_zero_grads": ([_P], _I),
            "tg3_cnn_adam": ([_P, ctypes.c_float], _I),
            "tg3_cnn_propose": ([_P, _I, _I, _I, ctypes.c_ulonglong, _P, _P, _P], _I),
            "tg3_cnn_backward": ([_P, _P, _I, _P], _I),
            "tg3_cnn_infer": ([_P, _P, _I, _P], _I),
            "tg3_cnn_contrastive": ([_P, _P, _P, _I, _P, _F, _P, _P, _P], _I),
            "tg3_cnn_embed": ([_P, _I, _P, _P], _I),
            "tg3_cnn_match_propose": ([_P, _I, _P, _I, _P, _I, _I, ctypes.c_ulonglong, _P, _P,
                                       _P, _P], _I),
            "tg3_ctx_set_bank": ([_P, _I, _P, _I], _I),
            "tg3_local_phase_ctf_d": ([_P, _I, _I, _I, _I] + [_P] * 16 + [_I], _I),
            "tg3_ExpectGlobal2D": ([_P] * 13 + [_I] * 9, _I),
            "tg3_InsertI2D": ([_P] * 16 + [_F] + [_I] * 8, _I),
            "tg3_global_scan2d_classes_d": ([_P, _P] + [_I] * 6 + [_P] * 11 + [_I], _I),
            "tg3_prepare_images_d": ([_P, _P, _I, _I, _F, _I, _F, _P, _P], _I),
            "tg3_sigma_d": ([_P, _I, _I] + [_P] * 7 + [_I, _I, _I, _F, _F, _P, _P], _I),
            "tg3_ctx_reconstruct_d": ([_P, _P, _I, _I, _I, _I, _I, _F, _F, _P, _P], _I),
            "tg3_ctx_insert_load_d": ([_P, _P, _P], _I),
            "tg3_mrc_info": ([ctypes.c_char_p] + [_P] * 5, _I),
            "tg3_mrc_read": ([ctypes.c_char_p, _I, _I, _P], _I),
            "tg3_mrc_write": ([ctypes.c_char_p, _P, _I, _I, _I, _F, _I], _I),
            "tg3_thu_count": ([ctypes.c_char_p, _P], _I),
            "tg3_thu_read": ([ctypes.c_char_p, _I, _P, _P, _P, _I], _I),
            "tg3_thu_write": ([ctypes.c_char_p, _I, _P, _P, _P, _I], _I),
            "tg3_global_scan2d_d": ([_P, _P, _I, _I, _I, _I, _I] + [_P] * 12 + [_I], _I),
            "tg3_ExpectLocal3D_ctf": ([_P, _P, _P, _P, _F, _F, _F, _F, _P, _P, _P, _I, _I, _P, _I,
                                       _P, _I, _P, _I, _P, _P, _P, _D, _P, _P, _P, _P, _P, _P],
                                      _I),
            "tg3_local_phase_bank_d": ([_P, _I, _I, _I] + [_P] * 14 + [_I], _I),
            "tg3_ctx_stage_times": ([_P, _P, _P, _I], _I),
            "tg3_noalloc_scratch_bytes": ([], ctypes.c_size_t),
            "tg3_global_scan_d": ([_P, _I, _I, _I, _I] + [_P] * 12 + [_I], _I),
            "tg3_local_phase_noalloc": ([_P, _I, _I, _P, _P, _I, _I, _P, _P, _P, _P, _I, _P, _I,
                                         _P, _P, _P, _P, _P, _P, _P, _P, _P], _I),
            "tg3_ctx_set_references": ([_P, _I, _P, _I], _I),
            "tg3_learned_expect_d": ([_P, _P, _I, _P, _P, _P, _P, _P, _I, _I,
                                      ctypes.c_ulonglong, _P, _I, _F, _I,
                                      ctypes.POINTER(LearnedOut)], _I),
            "tg3_ExpectLearned3D": ([_P, _P, _I, _P, _P, _P, _P, _P, _I, _I, ctypes.c_ulonglong,
                                     _P, _I, _F, _I, _P, _P, _P, _P, _P], _I),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def check(status: int):
    if status != OK:
        msg = lib().tg3_last_error().decode(errors="replace")
        raise TG3Error(status, msg)


def ptr(x) -> int | None:
    """Address of a torch tensor (device or host) or a numpy array; None -> 0."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return x.data_ptr()
    raise TypeError(type(x))



def fsc(A, B, n_shell: int, stream=None):
    """Fourier shell correlation of two complex half volumes on the device
    ([vdim][vdim][vdim/2+1], complex64 or float32 pairs): a float64 tensor of
    n_shell values, shells rint(|k|) in voxel units."""
    import torch
    vdim = A.shape[0]
    out = torch.empty(n_shell, dtype=torch.float64, device=A.device)
    scratch = torch.empty(3 * n_shell, dtype=torch.float64, device=A.device)
    check(lib().tg3_fsc_d(ptr(A), ptr(B), vdim, n_shell, ptr(out), ptr(scratch), stream))
    if stream is None:
        torch.cuda.synchronize(A.device)
    return out

class Context:
    """A tg3_ctx: stream, volumes, pixel list, workspace on one device.

    Device work is asynchronous on the context's stream, so every tensor
    passed to a method is kept alive until the next sync()."""

    def __init__(self, device: int = 0):
        h = ctypes.c_void_p()
        check(lib().tg3_ctx_create(ctypes.byref(h), device))
        self.h = h
        self.device = device
        self._keep = []

    def _hold(self, *xs):
        self._keep.extend(x for x in xs if x is not None and not isinstance(x, (int, float)))

    def close(self):
        if self.h:
            lib().tg3_ctx_destroy(self.h)
            self.h = None
        self._keep = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return lib().tg3_ctx_stream(self.h)

    def sync(self):
        check(lib().tg3_ctx_sync(self.h))
        self._keep = []

    def workspace_bytes(self) -> int:
        return lib().tg3_ctx_workspace_bytes(self.h)

    def set_volume(self, cls, vol, pf):
        """vol: complex64 tensor/array (vdim, vdim, vdim//2+1), host or device."""
        on_dev = int(hasattr(vol, "is_cuda") and vol.is_cuda)
        check(lib().tg3_ctx_set_volume(self.h, cls, ptr(vol), vol.shape[0], pf, on_dev))

    def set_pixels(self, iCol, iRow, idim):
        iCol = np.ascontiguousarray(iCol, np.int32)
        iRow = np.ascontiguousarray(iRow, np.int32)
        check(lib().tg3_ctx_set_pixels(self.h, ptr(iCol), ptr(iRow), len(iCol), idim))

    def local_phase(self, nP, nR, nT, dat, ctf, sig, quat, trans, pwR, pwT, pwC, cls,
                    wC, wR, wT, base, dvp=None, precision=SCORE_FP32):
        self._hold(dat, ctf, sig, quat, trans, pwR, pwT, pwC, cls, wC, wR, wT, base, dvp)
        check(lib().tg3_local_phase_d(self.h, nP, nR, nT, ptr(dat), ptr(ctf), ptr(sig),
                                      ptr(quat), ptr(trans), ptr(pwR), ptr(pwT), ptr(pwC),
                                      ptr(cls), ptr(wC), ptr(wR), ptr(wT), ptr(base), ptr(dvp),
                                      precision))

    def local_phase_ctf(self, nP, nR, nT, nD, dat, ctfD, sig, quat, trans, pwR, pwT, pwD, pwC,
                        cls, wC, wR, wT, wD, base, dvp=None, precision=SCORE_FP32):
        """Local phase with nD defocus hypotheses per particle (ctfD [nP][nD][K])."""
        self._hold(dat, ctfD, sig, quat, trans, pwR, pwT, pwD, pwC, cls, wC, wR, wT, wD, base, dvp)
        check(lib().tg3_local_phase_ctf_d(self.h, nP, nR, nT, nD, ptr(dat), ptr(ctfD), ptr(sig),
                                          ptr(quat), ptr(trans), ptr(pwR), ptr(pwT), ptr(pwD),
                                          ptr(pwC), ptr(cls), ptr(wC), ptr(wR), ptr(wT), ptr(wD),
                                          ptr(base), ptr(dvp), precision))

    def set_bank(self, cls: int, quat, nB: int):
        """Project class `cls` at nB rotations (quat [nB][4] float64, device)
        once, over the active pixel set."""
        self._hold(quat)
        check(lib().tg3_ctx_set_bank(self.h, cls, ptr(quat), nB))

    def local_phase_bank(self, nP, nR, nT, dat, ctf, sig, bank_idx, trans, pwR, pwT, pwC, cls,
                         wC, wR, wT, base, dvp=None, precision=SCORE_FP32):
        """local_phase with the rotations given as rows bank_idx [nP][nR] (int32)
        of the classes' banks."""
        self._hold(dat, ctf, sig, bank_idx, trans, pwR, pwT, pwC, cls, wC, wR, wT, base, dvp)
        check(lib().tg3_local_phase_bank_d(self.h, nP, nR, nT, ptr(dat), ptr(ctf), ptr(sig),
                                           ptr(bank_idx), ptr(trans), ptr(pwR), ptr(pwT),
                                           ptr(pwC), ptr(cls), ptr(wC), ptr(wR), ptr(wT),
                                           ptr(base), ptr(dvp), precision))

    def set_references(self, cls: int, emb):
        """The network's normalised embeddings emb [nB][64] (device float32) of
        clean references at the rotations of class `cls`'s bank."""
        check(lib().tg3_ctx_set_references(self.h, cls, ptr(emb), emb.shape[0]))

    def learned_expect(self, net, images, dat, ctf, sig, cls, n_rot, n_trans, seed, g_trans,
                       peak_min, precision, out: dict):
        """The learned E-step (tg3_learned_expect_d) on device tensors; `out`
        maps LearnedOut field names to device tensors (bestQuat, bestTrans and
        baseL required).  Returns after the work has finished."""
        o = LearnedOut(**{k: ptr(v) for k, v in out.items() if v is not None})
        check(lib().tg3_learned_expect_d(self.h, net.h, images.shape[0], ptr(images), ptr(dat),
                                         ptr(ctf), ptr(sig), ptr(cls), n_rot, n_trans, seed,
                                         ptr(g_trans), g_trans.shape[0], float(peak_min),
                                         precision, ctypes.byref(o)))
        self._keep = []

    def learned_expect_host(self, net, images, dat, ctf, sig, cls, n_rot, n_trans, seed,
                            g_trans, peak_min, precision, best_quat, best_trans, base,
                            peak=None, fell_back=None):
        """tg3_ExpectLearned3D: the same with host arrays or tensors (inputs
        copied in, outputs copied out inside the call)."""
        check(lib().tg3_ExpectLearned3D(self.h, net.h, images.shape[0], ptr(images), ptr(dat),
                                        ptr(ctf), ptr(sig), ptr(cls), n_rot, n_trans, seed,
                                        ptr(g_trans), g_trans.shape[0], float(peak_min),
                                        precision, ptr(best_quat), ptr(best_trans), ptr(base),
                                        ptr(peak), ptr(fell_back)))

    def local_phase_host(self, nP, nR, nT, dat, ctf, sig, quat, trans, pwR, pwT, pwC, cls,
                         wC, wR, wT, base, dvp=None, precision=SCORE_FP32):
        """Host-buffer batched phase (arrays/tensors in host memory); returns
        after the outputs are in host memory."""
        check(lib().tg3_local_phase(self.h, nP, nR, nT, ptr(dat), ptr(ctf), ptr(sig), ptr(quat),
                                    ptr(trans), ptr(pwR), ptr(pwT), ptr(pwC), ptr(cls), ptr(wC),
                                    ptr(wR), ptr(wT), ptr(base), ptr(dvp), precision))

    def set_option(self, option: int, value: int):
        check(lib().tg3_ctx_set_option(self.h, option, int(value)))

    def set_pixels_slot(self, slot: int, iCol, iRow, idim: int):
        iCol = np.ascontiguousarray(iCol, dtype=np.int32)
        iRow = np.ascontiguousarray(iRow, dtype=np.int32)
        check(lib().tg3_ctx_set_pixels_slot(self.h, slot, ptr(iCol), ptr(iRow), len(iCol), idim))

    def use_pixels(self, slot: int):
        check(lib().tg3_ctx_use_pixels(self.h, slot))

    def set_timing(self, enable: bool):
        check(lib().tg3_ctx_set_timing(self.h, int(enable)))

    def stage_times(self, reset: bool = False):
        """{stage: (milliseconds, launches)} accumulated since the last reset."""
        ms = np.zeros(len(STAGES))
        n = np.zeros(len(STAGES), np.int32)
        check(lib().tg3_ctx_stage_times(self.h, ptr(ms), ptr(n), int(reset)))
        return {s: (float(ms[i]), int(n[i])) for i, s in enumerate(STAGES)}

    def global_scan(self, cls, nImg, nR, nT, dat, ctf, sig, rotmat, trans, pR, pT,
                    wC, wR, wT, base, dvp=None, precision=SCORE_FP32):
        self._hold(dat, ctf, sig, rotmat, trans, pR, pT, wC, wR, wT, base, dvp)
        check(lib().tg3_global_scan_d(self.h, cls, nImg, nR, nT, ptr(dat), ptr(ctf), ptr(sig),
                                      ptr(rotmat), ptr(trans), ptr(pR), ptr(pT), ptr(wC),
                                      ptr(wR), ptr(wT), ptr(base), ptr(dvp), precision))

    def global_scan2d(self, img, pf, nImg, nR, nT, dat, ctf, sig, rot, trans, pR, pT,
                      wC, wR, wT, base, dvp=None, precision=SCORE_FP32):
        """Global scan against one 2-D class image img (device, complex
        [vdim][vdim/2 + 1]) at in-plane rotations rot [nR][2] = (cos, sin)."""
        self._hold(img, dat, ctf, sig, rot, trans, pR, pT, wC, wR, wT, base, dvp)
        check(lib().tg3_global_scan2d_d(self.h, ptr(img), img.shape[-2], pf, nImg, nR, nT,
                                        ptr(dat), ptr(ctf), ptr(sig), ptr(rot), ptr(trans),
                                        ptr(pR), ptr(pT), ptr(wC), ptr(wR), ptr(wT), ptr(base),
                                        ptr(dvp), precision))

    def global_scan2d_classes(self, imgs, pf, nImg, nR, nT, dat, ctf, sig, rot, trans, pR, pT,
                              wC, wR, wT, base, precision=SCORE_FP32):
        """Global scan against every 2-D class image imgs (device, complex
        [nK][vdim][vdim/2 + 1]) in one pass, merged over the classes: wC
        [nImg][nK], wR [nImg][nK][nR], wT [nImg][nK][nT], base [nImg] (float32)."""
        self._hold(imgs, dat, ctf, sig, rot, trans, pR, pT, wC, wR, wT, base)
        check(lib().tg3_global_scan2d_classes_d(self.h, ptr(imgs), imgs.shape[0], imgs.shape[-2],
                                                pf, nImg, nR, nT, ptr(dat), ptr(ctf), ptr(sig),
                                                ptr(rot), ptr(trans), ptr(pR), ptr(pT), ptr(wC),
                                                ptr(wR), ptr(wT), ptr(base), precision))

    def prepare_images(self, img, mask_radius_px, dat, mask=True, std_n=0.0, stats=None):
        """Real-space images img (device float32 (n, N, N), file order) to the
        pixel data dat (device complex64 (n, K)) of the active pixel set."""
        n, N = img.shape[0], img.shape[-1]
        self._hold(img, dat, stats)
        check(lib().tg3_prepare_images_d(self.h, ptr(img), n, N, float(mask_radius_px),
                                         int(bool(mask)), float(std_n), ptr(dat), ptr(stats)))

    def sigma(self, cls, datM, datN, ctf, rotmat, trans, offset, group, n_group, r_sig,
              mask_radius, pixel_size, sig, sig_rcp, by_group=True):
        """Noise spectrum of the images at their best poses: sig / sig_rcp
        (device float64 (n_group, r_sig)); the active pixel set must be the
        shells below r_sig (tg3.io.spectrum_pixels)."""
        n = datM.shape[0]
        self._hold(datM, datN, ctf, rotmat, trans, offset, group, sig, sig_rcp)
        check(lib().tg3_sigma_d(self.h, cls, n, ptr(datM), ptr(datN), ptr(ctf), ptr(rotmat),
                                ptr(trans), ptr(offset), ptr(group), n_group, int(by_group),
                                r_sig, float(mask_radius), float(pixel_size), ptr(sig),
                                ptr(sig_rcp)))

    def remask(self, img_ft, mask_radius_px, out=None, edge_width=6.0):
        """Re-mask image transforms img_ft (device complex64 (n, N, N/2 + 1),
        centre at index 0) into out (a new tensor unless given)."""
        if out is None:
            import torch
            out = torch.empty_like(img_ft)
        self._hold(img_ft, out)
        check(lib().tg3_remask_d(self.h, ptr(img_ft), img_ft.shape[0], img_ft.shape[-2],
                                 float(mask_radius_px), float(edge_width), ptr(out)))
        return out

    def prepare_tf(self, sym_mats, max_radius, normalise=True):
        """Normalise (1 / T at the origin) and symmetrise the insertion
        accumulators in place; sym_mats: (nSym, 3, 3) rotations besides the
        identity (host), or None."""
        m = np.ascontiguousarray(np.zeros((0, 9)) if sym_mats is None else sym_mats,
                                 dtype=np.float64).reshape(-1, 9)
        check(lib().tg3_ctx_prepare_tf_d(self.h, ptr(m) if len(m) else None, len(m),
                                         int(max_radius), int(bool(normalise))))
        self.sync()

    def insert_load(self, F, T):
        """Accumulator <- F (complex64) and T (float32), device half grids."""
        self._hold(F, T)
        check(lib().tg3_ctx_insert_load_d(self.h, ptr(F), ptr(T)))

    def reconstruct(self, vol, max_radius, fsc=None, join_half=False, grid_corr=True,
                    kernel=None, a=1.9, alpha=15.0):
        """The map from the insertion accumulators into vol (device float32
        (N, N, N), centred); returns the number of balancing rounds."""
        kernel = KERNEL_TRILINEAR if kernel is None else kernel
        self._hold(vol, fsc)
        rounds = ctypes.c_int(0)
        check(lib().tg3_ctx_reconstruct_d(self.h, ptr(fsc), 0 if fsc is None else len(fsc),
                                          int(join_half), max_radius, int(grid_corr), kernel,
                                          float(a), float(alpha), ptr(vol), ctypes.byref(rounds)))
        return rounds.value

    def resample(self, nP, n, u, w, perm, u0, peak, nOut, src, wOut, top):
        self._hold(u, w, perm, u0, peak, src, wOut, top)
        check(lib().tg3_resample_d(self.h, nP, n, ptr(u), ptr(w), ptr(perm), ptr(u0), ptr(peak),
                                   nOut, ptr(src), ptr(wOut), ptr(top)))

    def insert_begin(self, vdim, pf):
        check(lib().tg3_ctx_insert_begin(self.h, vdim, pf))

    def insert(self, nP, dat, ctf, quat, trans, offset, w, kernel, O3D=None, counter=None):
        self._hold(dat, ctf, quat, trans, offset, w, O3D, counter)
        check(lib().tg3_insert_d(self.h, nP, ptr(dat), ptr(ctf), ptr(quat), ptr(trans),
                                 ptr(offset), ptr(w), kernel, ptr(O3D), ptr(counter)))

    def insert_read(self, F, T, accumulate=False):
        self._hold(F, T)
        check(lib().tg3_ctx_insert_read_d(self.h, ptr(F), ptr(T), int(accumulate)))

    def insert_ratio(self, V, floor=0.0):
        """V (complex64 half volume, device) = F / T where T > floor, else 0."""
        self._hold(V)
        check(lib().tg3_ctx_insert_ratio_d(self.h, ptr(V), float(floor)))

    def project(self, cls, rotmat, nR, out):
        self._hold(rotmat, out)
        check(lib().tg3_project_d(self.h, cls, ptr(rotmat), nR, ptr(out)))

    def render_references(self, cls, rotmat, n, img, out):
        """tg3_ctx_render_references_d: out [n][img][img] float32 (device)."""
        self._hold(rotmat, out)
        check(lib().tg3_ctx_render_references_d(self.h, cls, ptr(rotmat), n, img, ptr(out)))


def version() -> str:
    return lib().tg3_version().decode()


RAGGED_INPUTS = ("dat", "ctf", "sig", "quat", "trans", "pwR", "pwT", "pwC", "permR", "u0R",
                 "peakR", "permT", "u0T", "peakT")
RAGGED_OUTPUTS = ("wC", "base", "wR", "wT", "srcR", "wOutR", "srcT", "wOutT", "topR", "topT")


class RaggedPlan:
    """tg3_ragged_plan: a batch of particles with uneven hypothesis sets.

    cls, nR, nT: host int arrays (one entry per particle); inp / out: dicts
    of device tensors packed particle after particle (RAGGED_INPUTS /
    RAGGED_OUTPUTS, layouts as in thunder_gb300.h).  budget 0 autotunes."""

    def __init__(self, ctx: Context, cls, nR, nT, inp: dict, out: dict,
                 precision: int = SCORE_FP32, budget: int = 0, graph: bool = True):
        self.ctx = ctx
        self._keep = [inp, out]
        self.cls = np.ascontiguousarray(cls, dtype=np.int32)
        self.nR = np.ascontiguousarray(nR, dtype=np.int32)
        self.nT = np.ascontiguousarray(nT, dtype=np.int32)
        h = ctypes.c_void_p()
        args = [ptr(inp[k]) for k in RAGGED_INPUTS] + [ptr(out[k]) for k in RAGGED_OUTPUTS]
        check(lib().tg3_ragged_plan_create(ctx.h, len(self.cls), ptr(self.cls), ptr(self.nR),
                                           ptr(self.nT), *args, precision, int(budget),
                                           int(graph), ctypes.byref(h)))
        self.h = h

    def run(self):
        check(lib().tg3_ragged_plan_run(self.h))

    def info(self):
        w = ctypes.c_int()
        b = ctypes.c_size_t()
        check(lib().tg3_ragged_plan_info(self.h, ctypes.byref(w), ctypes.byref(b)))
        return w.value, b.value

    def kblock(self) -> int:
        """The K block of the plan's split-bf16 cross term (64 or 32)."""
        k = ctypes.c_int()
        check(lib().tg3_ragged_plan_kblock(self.h, ctypes.byref(k)))
        return k.value

    def project_group(self) -> int:
        """The projection's rotations per CTA in the plan (4, 8 or 16)."""
        g = ctypes.c_int()
        check(lib().tg3_ragged_plan_project_group(self.h, ctypes.byref(g)))
        return g.value

    def close(self):
        if self.h:
            lib().tg3_ragged_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Cnn:
    """tg3_cnn: the pose-proposal network (64 x 64 images -> 68 outputs)."""

    N_OUT = 68

    def __init__(self, device: int = 0, seed: int = 1):
        h = ctypes.c_void_p()
        check(lib().tg3_cnn_create(ctypes.byref(h), device, seed))
        self.h = h

    @property
    def n_params(self) -> int:
        return lib().tg3_cnn_param_count(self.h)

    def params(self) -> np.ndarray:
        a = np.empty(self.n_params, np.float32)
        check(lib().tg3_cnn_params(self.h, ptr(a), 0))
        return a

    def set_params(self, a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        check(lib().tg3_cnn_params(self.h, ptr(a), 1))

    def grads(self) -> np.ndarray:
        a = np.empty(self.n_params, np.float32)
        check(lib().tg3_cnn_grads(self.h, ptr(a)))
        return a

    def set_bf16(self, enable: bool):
        check(lib().tg3_cnn_set_bf16(self.h, int(enable)))

    def forward(self, img, out):
        """img: device float32 [n][64][64]; out: device float32 [n][68]."""
        check(lib().tg3_cnn_forward(self.h, ptr(img), img.shape[0], ptr(out)))

    def infer(self, img, out):
        """Inference forward (bf16 activations, tensor cores): as forward."""
        check(lib().tg3_cnn_infer(self.h, ptr(img), img.shape[0], ptr(out)))

    def loss(self, img, Rstar, tstar, grads: bool = True) -> float:
        v = ctypes.c_double()
        check(lib().tg3_cnn_loss(self.h, ptr(img), img.shape[0], ptr(Rstar), ptr(tstar),
                                 int(grads), ctypes.byref(v)))
        return v.value

    def zero_grads(self):
        check(lib().tg3_cnn_zero_grads(self.h))

    @staticmethod
    def propose(out, n_rot, n_trans, seed, quat, trans, stream=None):
        """Hypotheses from outputs (device tensors; quat [n][n_rot][4], trans
        [n][n_trans][2] float64), asynchronous on `stream` (an int handle)."""
        check(lib().tg3_cnn_propose(ptr(out), out.shape[0], n_rot, n_trans, seed, ptr(quat),
                                    ptr(trans), stream))

    def adam(self, lr: float):
        check(lib().tg3_cnn_adam(self.h, lr))

    def backward(self, img, d_out):
        """Add the gradient of a loss with d loss / d outputs = d_out [n][68]."""
        check(lib().tg3_cnn_backward(self.h, ptr(img), img.shape[0], ptr(d_out)))

    def contrastive(self, out_p, out_r, tstar, tau, d_p, d_r) -> float:
        """Matching loss of particles against their references (device
        tensors); fills d_p, d_r with d loss / d outputs; returns the loss."""
        v = ctypes.c_double()
        check(lib().tg3_cnn_contrastive(self.h, ptr(out_p), ptr(out_r), out_p.shape[0],
                                        ptr(tstar), float(tau), ptr(d_p), ptr(d_r),
                                        ctypes.byref(v)))
        return v.value

    @staticmethod
    def embed(out, z, stream=None):
        check(lib().tg3_cnn_embed(ptr(out), out.shape[0], ptr(z), stream))

    @staticmethod
    def match_propose(out, ref, ref_quat, n_rot, n_trans, seed, quat, trans, idx=None,
                      stream=None):
        """Rotations: the n_rot references of highest score (and their indices
        into idx [n][n_rot] int32 when given); translations as propose
        (device tensors; ref [nRef][64] normalised, ref_quat [nRef][4])."""
        check(lib().tg3_cnn_match_propose(ptr(out), out.shape[0], ptr(ref), ref.shape[0],
                                          ptr(ref_quat), n_rot, n_trans, seed, ptr(quat),
                                          ptr(trans), ptr(idx), stream))

    def close(self):
        if self.h:
            lib().tg3_cnn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
