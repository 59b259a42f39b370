"""ctypes binding of libbats_gb300.so (the C ABI declared in include/bats_gb300.h).

The library is loaded once per process. There is no fallback: if the shared library is missing or
CUDA is unavailable, every call raises, so a silent CPU path cannot stand in for the kernels.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libbats_gb300.so")

_lock = threading.Lock()
_lib = None

c_int, c_ll, c_float, c_double, c_size, c_vp = (ctypes.c_int, ctypes.c_longlong, ctypes.c_float,
                                                 ctypes.c_double, ctypes.c_size_t, ctypes.c_void_p)

# name -> (restype, argtypes)
SIGNATURES = {
    "bats_abi_version": (c_int, []),
    "bats_status_string": (ctypes.c_char_p, [c_int]),
    "bats_last_error": (ctypes.c_char_p, []),
    "bats_read_device_status": (c_int, [c_vp, c_int]),
    "bats_compute_pre_exps": (c_int, [c_vp, c_ll, c_float, c_float, c_vp, c_vp, c_vp]),
    "bats_sort_events_workspace_bytes": (c_size, [c_int, c_int, c_int]),
    "bats_sort_events": (c_int, [c_vp, c_int, c_int, c_int, c_float, c_float, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                 c_vp, c_int, c_vp, c_size, c_vp]),
    "bats_sort_events_counted": (c_int, [c_vp, c_vp, c_int, c_int, c_int, c_float, c_float, c_vp, c_vp, c_vp, c_vp,
                                         c_vp, c_vp, c_vp, c_int, c_vp, c_size, c_vp]),
    "bats_sort_events_counted_ordered": (c_int, [c_vp, c_vp, c_int, c_int, c_int, c_float, c_float, c_vp, c_vp,
                                                 c_vp, c_vp, c_vp, c_vp, c_vp, c_int, c_vp, c_vp, c_size, c_vp]),
    "bats_sample_order": (c_int, [c_vp, c_int, c_vp, c_vp]),
    "bats_lif_forward_fc": (c_int, [c_vp, c_vp, c_ll, c_vp, c_int, c_int, c_int, c_int, c_float, c_float, c_float,
                                    c_float, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "bats_lif_forward_fc_default_algo": (c_int, [c_int, c_int, c_int]),
    "bats_lif_forward_fc_algo": (c_int, [c_vp, c_vp, c_ll, c_vp, c_int, c_int, c_int, c_int, c_float, c_float,
                                         c_float, c_float, c_vp, c_vp, c_vp, c_vp, c_vp, c_int, c_vp]),
    "bats_lif_forward_fc_queue_workspace_bytes": (c_size, [c_int]),
    "bats_lif_forward_fc_queue": (c_int, [c_vp, c_vp, c_ll, c_vp, c_int, c_int, c_int, c_int, c_float, c_float,
                                          c_float, c_float, c_vp, c_vp, c_vp, c_vp, c_vp, c_int, c_vp, c_size, c_vp]),
    "bats_intensity_to_spike_times": (c_int, [c_vp, c_int, c_int, ctypes.c_double, ctypes.c_double, c_vp, c_vp,
                                              c_vp]),
    "bats_nadam_step": (c_int, [c_vp, c_vp, c_vp, c_ll, c_float, c_float, c_float, c_float, ctypes.c_double,
                                ctypes.c_double, c_vp, c_vp]),
    "bats_weights_synaptic_scaling": (c_int, [c_vp, c_vp, c_vp, c_vp, c_int, c_int, c_int, c_float, c_float,
                                              c_vp]),
    "bats_label_weights_synaptic_scaling": (c_int, [c_vp, c_vp, c_vp, c_vp, c_int, c_int, c_int, c_float, c_vp]),
    "bats_conv_forward": (c_int, [c_vp, c_vp, c_ll, c_vp, c_int, c_int, c_int, c_int, c_int, c_int, c_int, c_int,
                                  c_float, c_float, c_float, c_float, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "bats_events_to_trains": (c_int, [c_vp, c_vp, c_int, c_int, c_int, c_int, c_vp, c_vp, c_vp, c_vp]),
    "bats_events_to_trains_csr": (c_int, [c_vp, c_vp, c_vp, c_int, c_int, c_int, c_vp, c_vp, c_vp, c_vp]),
    "bats_serve_fc_batch": (c_int, [c_vp, c_vp, c_vp, c_int, c_int, c_vp, c_vp, c_vp, c_int, c_int, c_vp, c_vp, c_vp,
                                    c_vp, c_int, c_vp, c_size, c_vp, c_vp, c_vp, c_vp]),
    "bats_events_max_per_neuron": (c_int, [c_vp, c_int, c_int, c_int, c_vp, c_vp, c_vp]),
    "bats_conv_backward_grouped": (c_int, [c_vp, c_vp, c_ll, c_vp, c_int, c_int, c_int, c_int, c_int, c_int, c_int,
                                           c_int, c_vp, c_vp, c_vp, c_int, c_float, c_float, c_vp, c_vp, c_vp]),
    "bats_pool_forward": (c_int, [c_vp, c_vp, c_int, c_int, c_int, c_int, c_int, c_vp, c_vp, c_vp, c_vp]),
    "bats_backward_prep": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_int, c_int, c_int, c_float, c_float, c_float,
                                   c_int, c_int, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "bats_cursor_heads_bytes": (c_size, [c_int, c_int]),
    "bats_backward_prep_counted": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_int, c_int, c_int, c_float, c_float,
                                           c_float, c_vp, c_vp, c_vp, c_vp]),
    "bats_backward_prep_layer": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_int, c_int, c_int, c_float, c_float, c_float,
                                         c_vp, c_vp, c_vp, c_vp, c_vp]),
    "bats_weights_gradient_workspace_bytes": (c_size, [c_int, c_int, c_int, c_int]),
    "bats_weights_gradient": (c_int, [c_vp, c_vp, c_vp, c_vp, c_ll, c_vp, c_vp, c_vp, c_vp, c_int, c_int, c_int,
                                      c_int, c_int, c_int, c_vp, c_vp, c_size, c_vp]),
    "bats_weights_gradient_adam": (c_int, [c_vp, c_vp, c_vp, c_vp, c_ll, c_vp, c_vp, c_vp, c_vp, c_int, c_int, c_int,
                                           c_int, c_int, c_vp, c_vp, c_vp, c_float, c_float, c_float, c_float, c_vp,
                                           c_vp, c_vp, c_int, c_vp, c_size, c_vp]),
    "bats_weights_gradient_noalloc_capacity": (c_ll, []),
    "bats_weights_gradient_mean_noalloc": (c_int, [c_vp, c_vp, c_ll, c_vp, c_vp, c_vp, c_int, c_int, c_int, c_int,
                                                   c_int, c_vp, c_vp]),
    "bats_pre_errors_workspace_bytes": (c_size, [c_int, c_ll, c_int]),
    "bats_pre_errors": (c_int, [c_vp, c_vp, c_vp, c_ll, c_vp, c_int, c_vp, c_vp, c_vp, c_int, c_int, c_int, c_int,
                                c_int, c_float, c_float, c_vp, c_vp, c_size, c_vp]),
    "bats_conv_backward": (c_int, [c_vp, c_vp, c_vp, c_ll, c_vp, c_int, c_int, c_int, c_int, c_int, c_int, c_int,
                                   c_int, c_vp, c_vp, c_vp, c_int, c_float, c_float, c_vp, c_vp, c_vp]),
    "bats_pool_backward": (c_int, [c_vp, c_vp, c_ll, c_vp, c_ll, c_vp]),
    "bats_spike_count_loss": (c_int, [c_vp, c_int, c_vp, c_vp, c_float, c_float, c_int, c_int, c_int, c_vp, c_vp,
                                      c_vp]),
    "bats_ttfs_softmax_cross_entropy": (c_int, [c_vp, c_vp, c_int, c_int, c_int, c_double, c_vp, c_vp, c_vp]),
    "bats_spike_time_loss": (c_int, [c_vp, c_vp, c_int, c_int, c_int, c_int, c_vp, c_vp, c_vp]),
    "bats_adam_step": (c_int, [c_vp, c_vp, c_vp, c_ll, c_float, c_float, c_float, c_float, c_double, c_double, c_vp,
                               c_vp, c_vp, c_int, c_int, c_int, c_vp]),
    "bats_adam_powers_advance": (c_int, [c_vp, c_float, c_float, c_vp]),
    "bats_adam_step_device": (c_int, [c_vp, c_vp, c_vp, c_ll, c_float, c_float, c_float, c_float, c_vp, c_vp, c_vp,
                                      c_int, c_int, c_int, c_vp]),
    "bats_add_deltas": (c_int, [c_vp, c_vp, c_ll, c_vp, c_int, c_int, c_vp]),
    "bats_transpose": (c_int, [c_vp, c_int, c_int, c_vp, c_int, c_vp]),
    "bats_copy_device": (c_int, [c_vp, c_vp, c_size, c_vp]),
    "bats_conv_backward_adam_workspace_bytes": (c_size, [c_int, c_int, c_int, c_int, c_int, c_int]),
    "bats_conv_backward_adam": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_ll, c_vp, c_int, c_int, c_int, c_int, c_int,
                                        c_int, c_int, c_int, c_vp, c_vp, c_vp, c_int, c_float, c_float, c_vp, c_int,
                                        c_vp, c_vp, c_vp, c_float, c_float, c_float, c_float, c_vp, c_vp, c_size,
                                        c_vp]),
    "bats_fc_train_step_workspace_bytes": (c_size, [c_int, c_vp, c_int]),
    "bats_fc_train_step": (c_int, [c_vp, c_vp, c_int, c_vp, c_int, c_float, c_float, c_float, c_float, c_float,
                                   c_float, c_vp, c_vp, c_vp, c_vp, c_size, c_vp]),
}


class BatsError(RuntimeError):
    """A non-zero status returned by the C ABI."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def load():
    """Load libbats_gb300.so and bind the signatures; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA library first "
                               "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


class BatsFcLayer(ctypes.Structure):
    """struct BatsFcLayer of include/bats_gb300.h (one layer of bats_serve_fc_batch)."""
    _fields_ = [("n_pre", c_int), ("k_pre", c_int), ("n_post", c_int), ("k_post", c_int), ("weights_t", c_vp),
                ("ld", c_int), ("tau_s", c_float), ("tau", c_float), ("c", c_float), ("delta_theta_tau", c_float),
                ("max_simulation", c_float), ("algo", c_int), ("events", c_vp), ("slots", c_vp),
                ("ev_count", c_vp), ("n_spikes", c_vp), ("a", c_vp), ("x", c_vp), ("times", c_vp),
                ("post_exp_tau", c_vp)]


class BatsFcTrainLayer(ctypes.Structure):
    """struct BatsFcTrainLayer of include/bats_gb300.h (one layer of bats_fc_train_step)."""
    _fields_ = [("fwd", BatsFcLayer), ("weights", c_vp), ("adam_m", c_vp), ("adam_v", c_vp), ("grad", c_vp),
                ("events_bucketed", c_vp), ("bucket_offsets", c_vp), ("tables", c_vp), ("nvalid", c_vp),
                ("cursor_heads", c_vp), ("f1", c_vp), ("f2", c_vp), ("pre_errors", c_vp), ("grad_group", c_int)]


def call(name: str, *args):
    """Call an entry point and raise BatsError on a non-zero status."""
    status = getattr(load(), name)(*args)
    if status != 0:
        msg = load().bats_last_error().decode(errors="replace")
        raise BatsError(status, f"{name} failed: {msg}")
    return status


def check_device_status() -> None:
    """Raise if a device-side bounded wait gave up since the last check (synchronising call)."""
    out = ctypes.c_int(0)
    call("bats_read_device_status", ctypes.byref(out), 1)


def ptr(t) -> int | None:
    """Device pointer of a tensor (None passes NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("bats_gb300 kernels take CUDA tensors")
    return t.data_ptr()


def stream_ptr(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("bats_gb300 needs a CUDA device; there is no CPU fallback")
