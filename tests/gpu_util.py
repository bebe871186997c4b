"""Device-buffer helpers for the GPU tests (torch tensors as plain device
memory; every computation goes through the C ABI)."""
import numpy as np

_DT = {np.dtype(np.int32): "int32", np.dtype(np.uint8): "uint8", np.dtype(np.uint32): "int32",
       np.dtype(np.uint64): "int64", np.dtype(np.int64): "int64"}


def torch():
    import torch as t

    return t


# Every buffer handed out stays referenced until release(): a raw pointer
# whose tensor was dropped would be recycled by torch's caching allocator and
# alias the next buffer.
_LIVE = []


def release():
    _LIVE.clear()


def dev(a: np.ndarray, pad: int = 0):
    """Copies a numpy array to a fresh device buffer (optionally with `pad`
    leading bytes so the data pointer is misaligned); returns (tensor, ptr)."""
    t = torch()
    raw = np.ascontiguousarray(a).view(np.uint8)
    buf = t.empty(raw.size + pad + 16, dtype=t.uint8, device="cuda")
    if raw.size:
        buf[pad:pad + raw.size].copy_(t.from_numpy(raw.copy()))
    _LIVE.append(buf)
    return buf, buf.data_ptr() + pad


def zeros(n: int, dtype, pad: int = 0):
    return dev(np.zeros(n, dtype), pad)


def host(buf, ptr, n, dtype):
    t = torch()
    t.cuda.synchronize()
    off = ptr - buf.data_ptr()
    nb = n * np.dtype(dtype).itemsize
    return buf[off:off + nb].cpu().numpy().view(dtype).copy()


def stream():
    return torch().cuda.current_stream().cuda_stream
