"""Device-memory entry points on torch tensors (uint64 stored as int64).

torch provides the device allocations and the stream; the arithmetic runs in
libhg_gb300.so.  Tensors must be contiguous int64 CUDA tensors holding the
64-bit limbs bit for bit.
"""

from __future__ import annotations

from ._lib import check, load


def _stream(stream):
    if stream is None:
        import torch

        return torch.cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


def _p(t):
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return t.data_ptr()


def mul(x, y, out, nx=None, ny=None, stream=None) -> None:
    """|x| * |y| into out (hg_mul_device); sizes default to the tensor lengths."""
    nx = x.numel() if nx is None else nx
    ny = y.numel() if ny is None else ny
    check(load().hg_mul_device(_p(x), nx, _p(y), ny, _p(out), out.numel(), _stream(stream)))


def sqr(x, out, nx=None, stream=None) -> None:
    nx = x.numel() if nx is None else nx
    check(load().hg_sqr_device(_p(x), nx, _p(out), out.numel(), _stream(stream)))


NOALLOC_MAX_LIMBS = 65536


def mul_noalloc(x, y, out, nx=None, ny=None, stream=None) -> None:
    """|x| * |y| (|x|^2 when y is None) into out on the library's fixed
    scratch (hg_mul_device_noalloc): no allocation, at most
    NOALLOC_MAX_LIMBS product limbs, calls on one stream at a time."""
    nx = x.numel() if nx is None else nx
    ny = (nx if y is None else y.numel()) if ny is None else ny
    yp = None if y is None else _p(y)
    check(load().hg_mul_device_noalloc(_p(x), nx, yp, ny, _p(out), out.numel(), _stream(stream)))


def mul_schoolboy(x, y, out, stream=None) -> None:
    check(load().hg_mul_schoolboy_device(_p(x), x.numel(), _p(y), y.numel(), _p(out), out.numel(), _stream(stream)))


def ntt_forward(a, mod_num: int, stream=None) -> None:
    """ntt-forward in place (bit-reversed output)."""
    check(load().hg_ntt_forward_device(_p(a), a.numel(), mod_num, _stream(stream)))


def ntt_reverse(a, mod_num: int, stream=None) -> None:
    """ntt-reverse in place (bit-reversed input, natural output, 1/N)."""
    check(load().hg_ntt_reverse_device(_p(a), a.numel(), mod_num, _stream(stream)))


def sync(stream=None) -> None:
    """Wait and surface device-side errors (hg_sync)."""
    check(load().hg_sync(None if stream is None else _stream(stream)))


def _products(items):
    """hg_product array from (x, y_or_None, out[, nx, ny]) tensor tuples."""
    from ._lib import HgProduct

    arr = (HgProduct * len(items))()
    for k, it in enumerate(items):
        x, y, out = it[0], it[1], it[2]
        nx = it[3] if len(it) > 3 and it[3] is not None else x.numel()
        ny = (it[4] if len(it) > 4 and it[4] is not None else y.numel()) if y is not None else 0
        arr[k] = HgProduct(_p(x), nx, None if y is None else _p(y), ny, _p(out), out.numel())
    return arr


class Batch:
    """A planned batch of products (hg_batch_create); run() enqueues it on a
    stream and can be captured in a CUDA graph.  Keeps the tensors alive."""

    def __init__(self, items, autotune: bool = True, schedule: str | None = None):
        """schedule: None (the persistent launch, or with autotune the faster
        of the two), "persistent" or "per_pass"."""
        import ctypes

        from ._lib import HG_BATCH_AUTOTUNE, HG_BATCH_PER_PASS, HG_BATCH_PERSISTENT

        flags = HG_BATCH_AUTOTUNE if autotune else 0
        if schedule == "persistent":
            flags |= HG_BATCH_PERSISTENT
        elif schedule == "per_pass":
            flags |= HG_BATCH_PER_PASS
        elif schedule is not None:
            raise ValueError(f"unknown schedule {schedule!r}")
        self._items = list(items)
        self._arr = _products(self._items)
        h = ctypes.c_void_p()
        check(load().hg_batch_create(self._arr, len(self._items), flags, ctypes.byref(h)))
        self._h = h

    def run(self, stream=None) -> None:
        check(load().hg_batch_run(self._h, _stream(stream)))

    def schedule(self) -> tuple[str, int]:
        """("persistent" or "per_pass", kernel launches per run)."""
        import ctypes

        pers, n = ctypes.c_int(), ctypes.c_size_t()
        check(load().hg_batch_schedule(self._h, ctypes.byref(pers), ctypes.byref(n)))
        return ("persistent" if pers.value else "per_pass"), n.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            load().hg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def mul_batch(items, stream=None) -> None:
    """One-shot batch (hg_mul_batch_device): items are (x, y_or_None, out)."""
    arr = _products(items)
    check(load().hg_mul_batch_device(arr, len(items), _stream(stream)))


# numpy view of hg_product records (six 64-bit fields), for bulk submission
PRODUCT_FIELDS = ("x", "nx", "y", "ny", "out", "nout")


def product_records(x_ptr, nx, y_ptr, ny, out_ptr, nout):
    """An (n, 6) uint64 array laid out as hg_product[n] from equal-length
    arrays of device addresses and sizes (y_ptr 0 squares x)."""
    import numpy as np

    cols = [np.asarray(c, dtype=np.uint64) for c in (x_ptr, nx, y_ptr, ny, out_ptr, nout)]
    return np.ascontiguousarray(np.stack(cols, axis=1))


class Service:
    """The device-resident multiply service (hg_svc_*): products on device
    memory, continuous batching on `slots` streams, admission by workspace."""

    def __init__(self, workspace_bytes: int = 0, slots: int = 2, max_batch: int = 0):
        import ctypes

        h = ctypes.c_void_p()
        check(load().hg_svc_open(workspace_bytes, slots, max_batch, ctypes.byref(h)))
        self._h = h

    def submit(self, items) -> list[int]:
        """Queue (x, y_or_None, out[, nx, ny]) tensor tuples; returns their tickets."""
        arr = _products(items)
        return self._submit_ptr(arr, len(items))

    def submit_records(self, rec) -> range:
        """Queue an (n, 6) uint64 hg_product record array (product_records)."""
        import ctypes

        from ._lib import HgProduct

        n = rec.shape[0]
        return self._submit_ptr(rec.ctypes.data_as(ctypes.POINTER(HgProduct)), n)

    def _submit_ptr(self, arr, n):
        import ctypes

        first = ctypes.c_uint64()
        check(load().hg_svc_submit(self._h, arr, n, ctypes.byref(first)))
        return range(first.value, first.value + n)

    def status(self, ticket: int) -> int:
        return load().hg_svc_status(self._h, ticket)

    def wait(self, ticket: int, timeout: float = -1.0) -> None:
        check(load().hg_svc_wait(self._h, ticket, timeout))

    def wait_all(self, timeout: float = -1.0) -> None:
        check(load().hg_svc_wait_all(self._h, timeout))

    def stats(self, reset: bool = False) -> dict:
        import ctypes

        from ._lib import HgSvcStats

        st = HgSvcStats()
        check(load().hg_svc_stats(self._h, ctypes.byref(st), 1 if reset else 0))
        return {name: getattr(st, name) for name, _ in HgSvcStats._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None):
            h, self._h = self._h, None
            check(load().hg_svc_close(h))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
