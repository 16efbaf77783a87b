"""Neural radiance cache (hash grid + MLP) over the C ABI.

    cache = NeuralRadianceCache(scene_lo, scene_hi)
    pred = cache.query(records)            # float32 [n, 13] CUDA -> [n, 3]
    loss = cache.train_step(records, targets)
    pass_.set_nrc(cache, train=True)       # attach to a WavefrontPathTracer
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import check

CONFIG_KEYS = ("n_levels", "features_per_level", "log2_table_size", "base_resolution",
               "max_resolution", "hidden_layers", "learning_rate", "beta1", "beta2", "epsilon",
               "loss_scale", "batch_size", "train_pixel_stride", "seed", "tensor_cores",
               "termination_spread", "ema_decay")


RECORD_FLOATS = 13   # position 3, normal 3, roughness 1, albedo 3, outgoing direction 3


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _check_records(records: torch.Tensor) -> None:
    if records.dim() != 2 or records.shape[1] != RECORD_FLOATS or records.dtype != torch.float32:
        raise ValueError(f"records must be float32 [n, {RECORD_FLOATS}], got "
                         f"{records.dtype} {tuple(records.shape)}")


class NeuralRadianceCache:
    def __init__(self, scene_lo, scene_hi, **config):
        self.lib = _lib.load()
        self.cfg = _lib.NrcConfig()
        self.lib.krr_nrc_config_default(C.byref(self.cfg))
        for k, v in config.items():
            if k not in CONFIG_KEYS:
                raise KeyError(k)
            setattr(self.cfg, k, type(getattr(self.cfg, k))(v))
        self.cfg.scene_lo[:] = [float(x) for x in scene_lo]
        self.cfg.scene_hi[:] = [float(x) for x in scene_hi]
        self._h = C.c_void_p()
        check(self.lib.krr_nrc_create(C.byref(self.cfg), C.byref(self._h)), "krr_nrc_create")

    def status(self) -> tuple[int, bool]:
        """(error flags of the cache's kernels since the last call, diverged):
        a diverged cache (a non-finite training loss) stops training and the
        pass renders as the plain tracer until new parameters are loaded."""
        flags, div = C.c_uint32(), C.c_int32()
        check(self.lib.krr_nrc_status(self._h, C.byref(flags), C.byref(div), _stream()),
              "krr_nrc_status")
        return int(flags.value), bool(div.value)

    def save(self, path: str) -> None:
        """Checkpoint: weights, hash table, Adam moments and step to a file."""
        check(self.lib.krr_nrc_save(self._h, str(path).encode()), "krr_nrc_save")

    def load(self, path: str) -> None:
        check(self.lib.krr_nrc_load(self._h, str(path).encode()), "krr_nrc_load")

    def info(self) -> _lib.NrcInfo:
        i = _lib.NrcInfo()
        check(self.lib.krr_nrc_info(self._h, C.byref(i)), "krr_nrc_info")
        return i

    def query(self, records: torch.Tensor) -> torch.Tensor:
        _check_records(records)
        records = records.contiguous()
        out = torch.empty((records.shape[0], 3), dtype=torch.float32, device="cuda")
        check(self.lib.krr_nrc_query(self._h, records.data_ptr(), records.shape[0], out.data_ptr(),
                                     _stream()), "krr_nrc_query")
        return out

    def train_step(self, records: torch.Tensor, targets: torch.Tensor) -> float:
        _check_records(records)
        loss = C.c_float()
        check(self.lib.krr_nrc_train_step(self._h, records.contiguous().data_ptr(),
                                          targets.contiguous().data_ptr(), records.shape[0],
                                          C.byref(loss), _stream()), "krr_nrc_train_step")
        return loss.value

    def params(self, which: int) -> np.ndarray:
        i = self.info()
        n = i.n_params_mlp if which % 2 == 0 else i.n_table_entries * 2
        out = np.empty(n, np.float32)
        check(self.lib.krr_nrc_get_params(self._h, which, out.ctypes.data, n), "get_params")
        return out

    def set_params(self, which: int, values: np.ndarray):
        v = np.ascontiguousarray(values, np.float32)
        check(self.lib.krr_nrc_set_params(self._h, which, v.ctypes.data, v.size), "set_params")

    def gradients(self, records: torch.Tensor, targets: torch.Tensor):
        i = self.info()
        gm = np.empty(i.n_params_mlp, np.float32)
        gt = np.empty(i.n_table_entries * 2, np.float32)
        loss = C.c_float()
        check(self.lib.krr_nrc_gradients(self._h, records.contiguous().data_ptr(),
                                         targets.contiguous().data_ptr(), records.shape[0],
                                         gm.ctypes.data, gt.ctypes.data, C.byref(loss)),
              "krr_nrc_gradients")
        return gm, gt, loss.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.krr_nrc_destroy(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
