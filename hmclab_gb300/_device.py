"""Device plumbing: CUDA availability, tensor conversion, stream handles."""
import numpy as _np

from hmclab_gb300 import _lib
from hmclab_gb300.Helpers.CustomExceptions import DeviceUnavailableError

try:
    import torch as _torch
except ImportError:  # pragma: no cover - torch is a hard requirement on GPU hosts
    _torch = None

DTYPES = {"float32": _lib.HMC_F32, "float64": _lib.HMC_F64}


def require_cuda():
    """Load the library and check that a CUDA device is usable."""
    if _torch is None or not _torch.cuda.is_available():
        raise DeviceUnavailableError("hmclab_gb300 needs a CUDA device; none is available (no CPU fallback)")
    _lib.load()
    return _torch.device("cuda", _torch.cuda.current_device())


def torch_dtype(dtype):
    return {"float32": _torch.float32, "float64": _torch.float64}[dtype]


def dtype_code(dtype):
    try:
        return DTYPES[dtype]
    except KeyError:
        raise ValueError(f"dtype must be 'float32' or 'float64', got {dtype!r}")


def normalise_dtype(dtype):
    if dtype in (None, "float64", _np.float64, "f64", "double"):
        return "float64"
    if dtype in ("float32", _np.float32, "f32", "single"):
        return "float32"
    if _torch is not None and dtype is _torch.float64:
        return "float64"
    if _torch is not None and dtype is _torch.float32:
        return "float32"
    raise ValueError(f"unsupported dtype {dtype!r}")


def upload(array, dtype, device=None):
    """Copy a numpy array (any float type) to a contiguous device tensor."""
    device = device or require_cuda()
    a = _np.array(array, dtype=_np.float64, order="C", copy=True)
    return _torch.from_numpy(a).to(device=device, dtype=torch_dtype(dtype)).contiguous()


def upload_int32(array, device=None):
    device = device or require_cuda()
    a = _np.ascontiguousarray(_np.asarray(array, dtype=_np.int32))
    return _torch.from_numpy(a).to(device=device).contiguous()


def ptr(t):
    return None if t is None else t.data_ptr()


def stream_handle(stream=None):
    if stream is None:
        stream = _torch.cuda.current_stream()
    return stream.cuda_stream


def empty(shape, dtype, device=None):
    device = device or require_cuda()
    return _torch.empty(shape, dtype=torch_dtype(dtype) if isinstance(dtype, str) else dtype, device=device)


def zeros(shape, dtype, device=None):
    device = device or require_cuda()
    return _torch.zeros(shape, dtype=torch_dtype(dtype) if isinstance(dtype, str) else dtype, device=device)
