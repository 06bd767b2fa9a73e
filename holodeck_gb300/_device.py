"""Device-side state shared by the SAM path: tensors, cosmology upload, status word, workspaces.

PyTorch supplies device memory and streams; all arithmetic runs in the CUDA kernels of
``_build/libholodeck_gb300.so``.
"""

import contextlib
import ctypes

import numpy as np

from . import _native as N
from . import constants as C

_COSMO_CACHE = {}
_DC_TABLE_N = 8192


def torch():
    import torch as _t
    return _t


def device(dev=None):
    t = torch()
    if not t.cuda.is_available():
        raise N.NativeUnavailable("holodeck_gb300 needs a CUDA device; none is available")
    N.load()
    return t.device("cuda" if dev is None else dev)


def as_device(arr, dev=None, dtype=None):
    """Contiguous float64 (or `dtype`) CUDA tensor from a numpy array / tensor / scalar sequence."""
    t = torch()
    dtype = t.float64 if dtype is None else dtype
    dev = device(dev)
    if isinstance(arr, t.Tensor):
        return arr.to(device=dev, dtype=dtype).contiguous()
    return t.as_tensor(np.ascontiguousarray(arr), dtype=dtype, device=dev)


def is_torch(x):
    try:
        import torch as _t
    except ImportError:   # pragma: no cover
        return False
    return isinstance(x, _t.Tensor)


def to_host(t):
    return t.detach().cpu().numpy()


class StatusWord:
    """A device int32 the kernels OR HGB_STATUS_* bits into."""

    def __init__(self, dev=None):
        t = torch()
        self.t = t.zeros(1, dtype=t.int32, device=device(dev))

    def reset(self):
        self.t.zero_()

    @property
    def ptr(self):
        return N.ptr(self.t)

    def read(self):
        return int(self.t.item())


def comoving_distance_table(cosmo, n=_DC_TABLE_N):
    """Values and u-derivatives of D_C on u = k/n, u = sqrt(1/(1+z)), for cubic Hermite lookup."""
    uu = np.arange(n + 1, dtype=np.float64) / n
    half = 0.5 * (1.0 - uu)
    mid = 0.5 * (1.0 + uu)
    nodes = mid[:, None] + half[:, None] * cosmo.gl_nodes
    integ = 2.0 / np.sqrt(cosmo.Om0 + cosmo.Ode0 * nodes ** 6)
    val = cosmo.hubble_distance * half * np.sum(integ * cosmo.gl_weights, axis=-1)
    der = -2.0 * cosmo.hubble_distance / np.sqrt(cosmo.Om0 + cosmo.Ode0 * uu ** 6)
    return val, der


def distance_ratio_table(cosmo, val, der, n=_DC_TABLE_N):
    """The FP32 entry points' distance table: g(u) = D_C(u) / (D_H (1 - u)) and dg/du on u = k/n, from
    the FP64 values and derivatives of :func:`comoving_distance_table`.  At u = 1 (z = 0) g is the
    limit -D_C'(1) / D_H = 2 / sqrt(Om0 + Ode0) and dg/du = -D_C''(1) / (2 D_H) = -3 Ode0 (Om0 + Ode0)^(-3/2)."""
    uu = np.arange(n + 1, dtype=np.float64) / n
    w = 1.0 - uu
    dh = cosmo.hubble_distance
    g = np.empty(n + 1)
    dg = np.empty(n + 1)
    g[:n] = val[:n] / (dh * w[:n])
    dg[:n] = (der[:n] * w[:n] + val[:n]) / (dh * w[:n] ** 2)
    s = cosmo.Om0 + cosmo.Ode0
    g[n] = 2.0 / np.sqrt(s)
    dg[n] = -3.0 * cosmo.Ode0 * s ** -1.5
    return g.astype(np.float32), dg.astype(np.float32)


class DeviceCosmology:
    """Device copies of a :class:`holodeck_gb300.cosmology.Cosmology` and its ``hgb_cosmo`` struct."""

    def __init__(self, cosmo, dev=None):
        self.cosmo = cosmo
        self.grid_z = as_device(cosmo._grid_z, dev)
        self.grid_age = as_device(cosmo._grid_age, dev)
        self.grid_dcom = as_device(cosmo._grid_dcom, dev)
        val, der = comoving_distance_table(cosmo)
        self.dc_val = as_device(val, dev)
        self.dc_der = as_device(der, dev)
        gv, gd = distance_ratio_table(cosmo, val, der)
        t = torch()
        self.dcg_val = as_device(gv, dev, dtype=t.float32)
        self.dcg_der = as_device(gd, dev, dtype=t.float32)
        s = N.HgbCosmo()
        s.H0 = cosmo.H0
        s.Om0 = cosmo.Om0
        s.Ode0 = cosmo.Ode0
        s.age_pref = 2.0 / (3.0 * cosmo.H0 * np.sqrt(cosmo.Ode0))
        s.age_c1 = np.sqrt(cosmo.Ode0 / cosmo.Om0)
        s.tz_c2 = 1.5 * cosmo.H0 * np.sqrt(cosmo.Ode0)
        s.age_limit = (cosmo._age_universe / C.GYR) * C.GYR
        s.hubble_distance = cosmo.hubble_distance
        s.grid_z = N.ptr(self.grid_z)
        s.grid_age = N.ptr(self.grid_age)
        s.grid_dcom = N.ptr(self.grid_dcom)
        s.grid_size = int(cosmo._grid_z.size)
        s.dc_val = N.ptr(self.dc_val)
        s.dc_der = N.ptr(self.dc_der)
        s.dc_n = _DC_TABLE_N
        s.dcg_val = N.ptr(self.dcg_val)
        s.dcg_der = N.ptr(self.dcg_der)
        self.struct = s
        # cached and used from every stream: the uploads are complete before the cache hands it out
        t.cuda.current_stream(device(dev)).synchronize()

    @property
    def ref(self):
        return ctypes.byref(self.struct)


def device_cosmology(cosmo, dev=None):
    dev = device(dev)
    key = (id(cosmo), str(dev))
    hit = _COSMO_CACHE.get(key)
    if hit is None or hit.cosmo is not cosmo:
        hit = DeviceCosmology(cosmo, dev)
        _COSMO_CACHE[key] = hit
    return hit


_SIDE_STREAMS = {}


def side_stream(role, dev=None, priority=0):
    """A second stream for grid stages that overlap the calling thread's current stream: one per
    (device, current stream, role), so host workers that each run on their own stream never share
    one.  ``priority`` -1 makes the block scheduler start this stream's blocks first as SMs free up
    (CUDA stream priorities; 0 is the default and lowest)."""
    t = torch()
    cur = t.cuda.current_stream(device(dev))
    key = (cur.device.index, cur.cuda_stream, role)
    s = _SIDE_STREAMS.get(key)
    if s is None:
        s = _SIDE_STREAMS.setdefault(key, t.cuda.Stream(device=cur.device, priority=int(priority)))
    return s


@contextlib.contextmanager
def nvtx(name):
    """An NVTX range named ``name`` around a stage (Nsight Systems timelines, ``ncu --nvtx``
    filters); a no-op where torch has no NVTX support."""
    try:
        torch().cuda.nvtx.range_push(name)
        pushed = True
    except Exception:   # no NVTX in this torch build
        pushed = False
    try:
        yield
    finally:
        if pushed:
            torch().cuda.nvtx.range_pop()


def workspace(nbytes, dev=None):
    """A byte buffer for an entry point's scratch memory (from torch's caching allocator)."""
    t = torch()
    nbytes = max(int(nbytes), 1)
    return t.empty(nbytes, dtype=t.uint8, device=device(dev))
