"""Loads libigr_gb300.so (built in-tree by build.py) and manages contexts.

There is no fallback: if the library cannot be loaded, every call raises.
"""
import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libigr_gb300.so")

STATUS = {0: "IGR_OK", 1: "IGR_EINVAL", 2: "IGR_EUNSUPPORTED", 3: "IGR_ENONFINITE", 4: "IGR_ECUDA", 5: "IGR_ENOMEM",
          6: "IGR_ETIMEOUT"}

_lib = None
_lock = threading.Lock()


class IGRError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError("libigr_gb300.so is not built; run igr_sensitivities_gb300/build.py "
                                   "(or __graft_entry__.build()) first")
            _lib = C.CDLL(LIB_PATH)
            _lib.igr_last_error.restype = C.c_char_p
            _lib.igr_last_error.argtypes = [C.c_void_p]
            _lib.igr_ctx_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
            _lib.igr_ctx_destroy.argtypes = [C.c_void_p]
            _lib.igr_set_tape_budget.argtypes = [C.c_void_p, C.c_size_t]
            _lib.igr_last_launch_count.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
            _lib.igr_set_autotune.argtypes = [C.c_void_p, C.c_int, C.c_char_p]
        return _lib


class Context:
    """One CUDA stream plus device workspace (igr_ctx). Not thread-safe."""

    def __init__(self, device=0):
        h = C.c_void_p()
        rc = lib().igr_ctx_create(int(device), C.byref(h))
        if rc != 0:
            raise IGRError(rc, "igr_ctx_create failed (no usable CUDA device %d?)" % device)
        self.handle = h

    def close(self):
        if self.handle:
            lib().igr_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tape_budget(self, nbytes):
        check(self, lib().igr_set_tape_budget(self.handle, C.c_size_t(int(nbytes))))

    def last_launch_count(self):
        n = C.c_longlong(0)
        check(self, lib().igr_last_launch_count(self.handle, C.byref(n)))
        return n.value

    def set_cluster_size_1d(self, cs):
        """1D: CTAs per instance (0 = automatic; 1, 2, 4, 8, 16)."""
        check(self, lib().igr_set_cluster_size_1d(self.handle, C.c_int(int(cs))))

    def set_graphs(self, on):
        """2D forward and tangent solves: replay repeated RK steps as CUDA graphs (default on)."""
        check(self, lib().igr_set_graphs(self.handle, C.c_int(1 if on else 0)))

    def set_pcg_persistent(self, on):
        """2D untaped PCG solves of one wave of tiles: one persistent launch per
        solve (default on) or two kernels per iteration; bitwise the same."""
        check(self, lib().igr_set_pcg_persistent(self.handle, C.c_int(1 if on else 0)))

    def test_pcg_drop_tile(self, tile):
        """Test hook: the next persistent PCG launch runs with one tile's CTA
        leaving early, so the call returns IGR_ETIMEOUT (6) after 1 s."""
        check(self, lib().igr_test_pcg_drop_tile(self.handle, C.c_int(int(tile))))

    def set_autotune(self, on, cache_path=None):
        """Measure result-invariant launch choices (1D CTAs per instance, 2D fused
        or separate PCG inner products) on the first call of each batch shape and
        keep the fastest; cache_path keeps them in a file across processes."""
        path = None if cache_path is None else os.fsencode(cache_path)
        check(self, lib().igr_set_autotune(self.handle, C.c_int(1 if on else 0), path))

    def autotune_count(self):
        n = C.c_int(0)
        check(self, lib().igr_autotune_count(self.handle, C.byref(n)))
        return n.value

    def last_cluster_size_1d(self):
        v = C.c_int(0)
        check(self, lib().igr_last_cluster_size_1d(self.handle, C.byref(v)))
        return v.value

    def last_adjoint_plan(self):
        """Memory plan of the last adjoint call: instance groups, instances per
        group, steps taped per segment and segments (recomputed from checkpoints)."""
        v = [C.c_int(0) for _ in range(4)]
        check(self, lib().igr_last_adjoint_plan(self.handle, *[C.byref(x) for x in v]))
        return dict(zip(("groups", "instances_per_group", "steps_per_segment", "segments"), (x.value for x in v)))

    def last_checkpoint_schedule(self):
        """2D discrete adjoint: RK steps taped at once, checkpoint slots beyond
        the initial state and RK step evaluations of its revolve schedule."""
        w, s, e = C.c_int(0), C.c_int(0), C.c_longlong(0)
        check(self, lib().igr_last_checkpoint_schedule(self.handle, C.byref(w), C.byref(s), C.byref(e)))
        return {"tape_steps": w.value, "snapshots": s.value, "step_evaluations": e.value}


_default = None


def default_context():
    global _default
    if _default is None:
        _default = Context(int(os.environ.get("IGR_DEVICE", "0")))
    return _default


def check(ctx, rc):
    if rc != 0:
        raise IGRError(rc, lib().igr_last_error(ctx.handle).decode())
