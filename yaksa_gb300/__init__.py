"""yaksa_gb300 -- Python binding of the GB300 pack/unpack engine (libyaksa.so).

The engine is a C library with the reference's public C API (include/yaksa.h); this
module binds that C-ABI with ctypes so tests and the bench drive exactly the entry
points a C caller (or MPICH) would.  Names and argument meaning follow the reference
API (src/frontend/include/yaksa.h.in:221-634); errors are raised as YaksaError with
the library's return code.

    import yaksa_gb300 as yk
    y = yk.Yaksa()                      # loads yaksa_gb300/lib/libyaksa.so
    y.init()
    t = y.type_create_hvector(1024, 4, 128, yk.TYPE_DOUBLE)
    nbytes = y.pack(src_ptr, 1, t, 0, dst_ptr, 32768)

There is no CPU fallback: if the library is missing, loading raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libyaksa.so")

# operators (yaksa.h.in:37-48)
OP_MAX, OP_MIN, OP_SUM, OP_PROD, OP_LAND, OP_BAND, OP_LOR, OP_BOR, OP_LXOR, OP_BXOR, \
    OP_REPLACE = range(11)
OP_NAMES = {"max": OP_MAX, "min": OP_MIN, "sum": OP_SUM, "prod": OP_PROD, "land": OP_LAND,
            "band": OP_BAND, "lor": OP_LOR, "bor": OP_BOR, "lxor": OP_LXOR, "bxor": OP_BXOR,
            "replace": OP_REPLACE}

# builtin handles (yaksa.h.in:67-139)
TYPE_NULL = 0
TYPE_BOOL = 1
TYPE_CHAR = 2
TYPE_WCHAR_T = 5
TYPE_INT8_T, TYPE_INT16_T, TYPE_INT32_T, TYPE_INT64_T = 6, 7, 8, 9
TYPE_UINT8_T, TYPE_UINT16_T, TYPE_UINT32_T, TYPE_UINT64_T = 10, 11, 12, 13
TYPE_INT, TYPE_UNSIGNED, TYPE_SHORT = 14, 15, 16
TYPE_LONG = 18
TYPE_BYTE = 38
TYPE_FLOAT, TYPE_DOUBLE, TYPE_LONG_DOUBLE = 45, 46, 47
TYPE_C_COMPLEX, TYPE_C_DOUBLE_COMPLEX, TYPE_C_LONG_DOUBLE_COMPLEX = 48, 49, 50
TYPE_FLOAT_INT, TYPE_DOUBLE_INT, TYPE_LONG_INT, TYPE_2INT, TYPE_SHORT_INT, \
    TYPE_LONG_DOUBLE_INT = 51, 52, 53, 54, 55, 56

SUBARRAY_ORDER_C, SUBARRAY_ORDER_FORTRAN = 0, 1

SUCCESS, ERR_OUT_OF_MEM, ERR_INTERNAL, ERR_NOT_SUPPORTED = 0, 1, 2, 3

_u64 = ctypes.c_uint64
_ip = ctypes.c_ssize_t
_up = ctypes.c_size_t
_vp = ctypes.c_void_p

_PROTOS = {
    "yaksa_init": (ctypes.c_int, [_vp]),
    "yaksa_finalize": (ctypes.c_int, []),
    "yaksa_info_create": (ctypes.c_int, [ctypes.POINTER(_vp)]),
    "yaksa_info_free": (ctypes.c_int, [_vp]),
    "yaksa_info_keyval_append": (ctypes.c_int, [_vp, ctypes.c_char_p, _vp, ctypes.c_uint]),
    "yaksa_type_create_vector": (ctypes.c_int, [_ip, _ip, _ip, _u64, _vp, ctypes.POINTER(_u64)]),
    "yaksa_type_create_hvector": (ctypes.c_int, [_ip, _ip, _ip, _u64, _vp, ctypes.POINTER(_u64)]),
    "yaksa_type_create_contig": (ctypes.c_int, [_ip, _u64, _vp, ctypes.POINTER(_u64)]),
    "yaksa_type_create_dup": (ctypes.c_int, [_u64, _vp, ctypes.POINTER(_u64)]),
    "yaksa_type_create_indexed_block": (ctypes.c_int, [_ip, _ip, ctypes.POINTER(_ip), _u64, _vp,
                                                        ctypes.POINTER(_u64)]),
    "yaksa_type_create_hindexed_block": (ctypes.c_int, [_ip, _ip, ctypes.POINTER(_ip), _u64, _vp,
                                                         ctypes.POINTER(_u64)]),
    "yaksa_type_create_indexed": (ctypes.c_int, [_ip, ctypes.POINTER(_ip), ctypes.POINTER(_ip), _u64,
                                                  _vp, ctypes.POINTER(_u64)]),
    "yaksa_type_create_hindexed": (ctypes.c_int, [_ip, ctypes.POINTER(_ip), ctypes.POINTER(_ip),
                                                   _u64, _vp, ctypes.POINTER(_u64)]),
    "yaksa_type_create_resized": (ctypes.c_int, [_u64, _ip, _ip, _vp, ctypes.POINTER(_u64)]),
    "yaksa_type_create_struct": (ctypes.c_int, [_ip, ctypes.POINTER(_ip), ctypes.POINTER(_ip),
                                                 ctypes.POINTER(_u64), _vp, ctypes.POINTER(_u64)]),
    "yaksa_type_create_subarray": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_ip),
                                                   ctypes.POINTER(_ip), ctypes.POINTER(_ip),
                                                   ctypes.c_int, _u64, _vp, ctypes.POINTER(_u64)]),
    "yaksa_type_get_size": (ctypes.c_int, [_u64, ctypes.POINTER(_up)]),
    "yaksa_type_get_extent": (ctypes.c_int, [_u64, ctypes.POINTER(_ip), ctypes.POINTER(_ip)]),
    "yaksa_type_get_true_extent": (ctypes.c_int, [_u64, ctypes.POINTER(_ip), ctypes.POINTER(_ip)]),
    "yaksa_type_free": (ctypes.c_int, [_u64]),
    "yaksa_request_test": (ctypes.c_int, [_u64, ctypes.POINTER(ctypes.c_int)]),
    "yaksa_request_wait": (ctypes.c_int, [_u64]),
    "yaksa_ipack": (ctypes.c_int, [_vp, _up, _u64, _up, _vp, _up, ctypes.POINTER(_up), _vp, _u64,
                                   ctypes.POINTER(_u64)]),
    "yaksa_pack": (ctypes.c_int, [_vp, _up, _u64, _up, _vp, _up, ctypes.POINTER(_up), _vp, _u64]),
    "yaksa_iunpack": (ctypes.c_int, [_vp, _up, _vp, _up, _u64, _up, ctypes.POINTER(_up), _vp, _u64,
                                     ctypes.POINTER(_u64)]),
    "yaksa_unpack": (ctypes.c_int, [_vp, _up, _vp, _up, _u64, _up, ctypes.POINTER(_up), _vp, _u64]),
    "yaksa_pack_stream": (ctypes.c_int, [_vp, _up, _u64, _up, _vp, _up, ctypes.POINTER(_up), _vp,
                                         _u64, _vp]),
    "yaksa_unpack_stream": (ctypes.c_int, [_vp, _up, _vp, _up, _u64, _up, ctypes.POINTER(_up), _vp,
                                           _u64, _vp]),
    "yaksa_iov_len": (ctypes.c_int, [_up, _u64, ctypes.POINTER(_up)]),
    "yaksa_iov_len_max": (ctypes.c_int, [_up, _u64, _up, ctypes.POINTER(_up), ctypes.POINTER(_up)]),
    "yaksa_iov": (ctypes.c_int, [_vp, _up, _u64, _up, _vp, _up, ctypes.POINTER(_up)]),
    "yaksa_flatten_size": (ctypes.c_int, [_u64, ctypes.POINTER(_up)]),
    "yaksa_flatten": (ctypes.c_int, [_u64, _vp]),
    "yaksa_unflatten": (ctypes.c_int, [ctypes.POINTER(_u64), _vp]),
}


class IoVec(ctypes.Structure):
    """struct iovec"""
    _fields_ = [("iov_base", _vp), ("iov_len", _up)]


class PupOp(ctypes.Structure):
    """yaksa_gb300_pup_t (include/yaksa_gb300.h): one request of a batch."""
    _fields_ = [("kind", ctypes.c_int32), ("pad", ctypes.c_int32), ("inbuf", _vp), ("outbuf", _vp),
                ("count", _up), ("type", _u64), ("offset", _up), ("maxbytes", _up), ("op", _u64),
                ("actual", _up)]


class Rows(ctypes.Structure):
    """yaksa_gb300_rows_t (include/yaksa_gb300.h): n1 x n0 runs of `run` bytes at
    base + i1 * s1 + i0 * s0, for the row-touch measurement instrument."""
    _fields_ = [("base", _vp), ("n1", _u64), ("s1", ctypes.c_int64), ("n0", _u64),
                ("s0", ctypes.c_int64), ("run", ctypes.c_uint32), ("pad", ctypes.c_uint32)]


def pack_op(inbuf, count, t, offset, outbuf, maxbytes, op=10):
    return PupOp(0, 0, inbuf, outbuf, count, t, offset, maxbytes, op, 0)


def unpack_op(inbuf, insize, outbuf, count, t, offset, op=10):
    return PupOp(1, 0, inbuf, outbuf, count, t, offset, insize, op, 0)


class YaksaError(RuntimeError):
    def __init__(self, fn, rc):
        super().__init__(f"{fn} returned {rc}")
        self.rc = rc


def load_library(path):
    """Load a library exporting the yaksa C ABI privately (RTLD_LOCAL), so the product
    and the CPU oracle can live in one process."""
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing; run `python -m yaksa_gb300.build`")
    lib = ctypes.CDLL(path, mode=os.RTLD_LOCAL | os.RTLD_NOW)
    for name, (res, args) in _PROTOS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if hasattr(lib, "yaksa_gb300_stats"):
        lib.yaksa_gb300_stats.restype = ctypes.c_int
        lib.yaksa_gb300_stats.argtypes = [ctypes.POINTER(_u64)] * 4
        lib.yaksa_gb300_shard.restype = ctypes.c_int
        lib.yaksa_gb300_shard.argtypes = [_u64, _up, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_up),
                                          ctypes.POINTER(_up)]
        lib.yaksa_gb300_debug_fail_alloc.restype = ctypes.c_int
        lib.yaksa_gb300_debug_fail_alloc.argtypes = [ctypes.c_int]
        lib.yaksa_gb300_autotune_stats.restype = ctypes.c_int
        lib.yaksa_gb300_autotune_stats.argtypes = [ctypes.POINTER(ctypes.c_uint32),
                                                   ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(_u64)]
        for name, extra in (("yaksa_gb300_pup_batch_stream", [_vp]), ("yaksa_gb300_pup_batch", []),
                            ("yaksa_gb300_ipup_batch", [ctypes.POINTER(_u64)])):
            f = getattr(lib, name)
            f.restype = ctypes.c_int
            f.argtypes = [ctypes.POINTER(PupOp), ctypes.c_int, _vp] + extra
        lib.yaksa_gb300_graph_create.restype = ctypes.c_int
        lib.yaksa_gb300_graph_create.argtypes = [ctypes.POINTER(PupOp), ctypes.POINTER(ctypes.c_int),
                                                 ctypes.c_int, _vp, ctypes.POINTER(_vp)]
        lib.yaksa_gb300_graph_launch.restype = ctypes.c_int
        lib.yaksa_gb300_graph_launch.argtypes = [_vp, _vp]
        lib.yaksa_gb300_graph_free.restype = ctypes.c_int
        lib.yaksa_gb300_graph_free.argtypes = [_vp]
        for name, args in (("yaksa_gb300_server_create", [ctypes.c_uint32, _u64, ctypes.POINTER(_vp)]),
                           ("yaksa_gb300_server_submit", [_vp, ctypes.POINTER(PupOp), _vp,
                                                          ctypes.POINTER(_u64)]),
                           ("yaksa_gb300_server_test", [_vp, _u64, ctypes.POINTER(ctypes.c_int)]),
                           ("yaksa_gb300_server_wait", [_vp, _u64]),
                           ("yaksa_gb300_server_progress", [_vp]),
                           ("yaksa_gb300_server_stats", [_vp, ctypes.POINTER(_u64), ctypes.POINTER(_u64),
                                                         ctypes.POINTER(_u64),
                                                         ctypes.POINTER(ctypes.c_uint32)]),
                           ("yaksa_gb300_server_destroy", [_vp]),
                           ("yaksa_gb300_server_tune", [_vp, ctypes.POINTER(PupOp), ctypes.c_int, _vp,
                                                        ctypes.POINTER(ctypes.c_int)]),
                           ("yaksa_gb300_pup_noalloc", [ctypes.POINTER(PupOp), _vp]),
                           ("yaksa_gb300_probe_rows", [ctypes.POINTER(Rows), ctypes.c_int, ctypes.c_int, _vp]),
                           ("yaksa_gb300_debug_hidx_shape", [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
                           ("yaksa_gb300_debug_l2_reduce", [ctypes.c_int, ctypes.POINTER(ctypes.c_ulonglong)]),
                           ("yaksa_gb300_graph_lane_stats", [ctypes.POINTER(_u64), ctypes.POINTER(_u64)]),
                           ("yaksa_gb300_serve_trace", [ctypes.POINTER(PupOp), ctypes.POINTER(ctypes.c_double),
                                                        ctypes.c_int, ctypes.c_int, _vp, _vp,
                                                        ctypes.POINTER(ctypes.c_double),
                                                        ctypes.POINTER(ctypes.c_double)])):
            f = getattr(lib, name)
            f.restype = ctypes.c_int
            f.argtypes = args
    return lib


class Server:
    """Persistent-kernel request server (yaksa_gb300_server_*)."""

    def __init__(self, y, ring_requests=4096, budget_bytes=0):
        self.y = y
        self.h = _vp()
        y._chk("yaksa_gb300_server_create",
               y.lib.yaksa_gb300_server_create(ring_requests, budget_bytes, ctypes.byref(self.h)))

    def submit(self, op, info=None):
        """Returns a ticket, or None when admission is refused (retry after progress)."""
        t = _u64()
        rc = self.y.lib.yaksa_gb300_server_submit(self.h, ctypes.byref(op), info, ctypes.byref(t))
        if rc == ERR_OUT_OF_MEM:
            return None
        self.y._chk("yaksa_gb300_server_submit", rc)
        return t.value

    def test(self, ticket):
        d = ctypes.c_int()
        self.y._chk("yaksa_gb300_server_test", self.y.lib.yaksa_gb300_server_test(self.h, ticket,
                                                                                  ctypes.byref(d)))
        return bool(d.value)

    def wait(self, ticket):
        self.y._chk("yaksa_gb300_server_wait", self.y.lib.yaksa_gb300_server_wait(self.h, ticket))

    def progress(self):
        self.y._chk("yaksa_gb300_server_progress", self.y.lib.yaksa_gb300_server_progress(self.h))

    def tune(self, ops, info=None):
        """yaksa_gb300_server_tune over an array of PupOp; returns the classes decided."""
        c = ctypes.c_int()
        self.y._chk("yaksa_gb300_server_tune",
                    self.y.lib.yaksa_gb300_server_tune(self.h, ops, len(ops), info, ctypes.byref(c)))
        return c.value

    def stats(self):
        a, b, c, d = _u64(), _u64(), _u64(), ctypes.c_uint32()
        self.y.lib.yaksa_gb300_server_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                            ctypes.byref(d))
        return dict(requests=a.value, items=b.value, relaunches=c.value, idle_exits=d.value)

    def destroy(self):
        if self.h:
            self.y._chk("yaksa_gb300_server_destroy", self.y.lib.yaksa_gb300_server_destroy(self.h))
            self.h = None


def serve_trace(y, ops, arrival_s, server=None, info=None, graphs=False):
    """Replay `ops` (a yaksa_gb300_pup_t array) arriving at `arrival_s` seconds through
    the plain nonblocking path (server None; with the graph lane for repeated requests
    when `graphs`) or `server`; returns (latencies, makespan)."""
    n = len(ops)
    arr = (ctypes.c_double * max(1, n))(*arrival_s)
    lat = (ctypes.c_double * max(1, n))()
    mk = ctypes.c_double()
    mode = 1 if server is not None else 2 if graphs else 0
    y._chk("yaksa_gb300_serve_trace",
           y.lib.yaksa_gb300_serve_trace(ops, arr, n, mode, server.h if server is not None else None,
                                         info, lat, ctypes.byref(mk)))
    return list(lat[:n]), mk.value


def _arr(ctype, seq):
    seq = list(seq)
    return (ctype * max(1, len(seq)))(*seq)


class Yaksa:
    """The reference's public API over one loaded library (product by default)."""

    def __init__(self, path=LIB_PATH):
        self.path = path
        self.lib = load_library(path)

    def _chk(self, fn, rc):
        if rc != SUCCESS:
            raise YaksaError(fn, rc)

    def init(self, info=None):
        self._chk("yaksa_init", self.lib.yaksa_init(info))

    def finalize(self):
        self._chk("yaksa_finalize", self.lib.yaksa_finalize())

    # info
    def info_create(self, **kv):
        h = _vp()
        self._chk("yaksa_info_create", self.lib.yaksa_info_create(ctypes.byref(h)))
        for k, v in kv.items():
            if isinstance(v, str):
                b = v.encode()
                buf = ctypes.create_string_buffer(b)
                rc = self.lib.yaksa_info_keyval_append(h, k.encode(), ctypes.cast(buf, _vp), len(b))
            else:
                c = ctypes.c_int(v)
                rc = self.lib.yaksa_info_keyval_append(h, k.encode(), ctypes.cast(ctypes.byref(c), _vp),
                                                       ctypes.sizeof(c))
            self._chk("yaksa_info_keyval_append", rc)
        return h

    def info_free(self, h):
        self._chk("yaksa_info_free", self.lib.yaksa_info_free(h))

    # constructors
    def _new(self, fn, *args):
        out = _u64()
        self._chk(fn, getattr(self.lib, fn)(*args, None, ctypes.byref(out)))
        return out.value

    def type_create_vector(self, count, bl, stride, old):
        return self._new("yaksa_type_create_vector", count, bl, stride, old)

    def type_create_hvector(self, count, bl, stride, old):
        return self._new("yaksa_type_create_hvector", count, bl, stride, old)

    def type_create_contig(self, count, old):
        return self._new("yaksa_type_create_contig", count, old)

    def type_create_dup(self, old):
        return self._new("yaksa_type_create_dup", old)

    def type_create_indexed_block(self, bl, displs, old):
        return self._new("yaksa_type_create_indexed_block", len(displs), bl, _arr(_ip, displs), old)

    def type_create_hindexed_block(self, bl, displs, old):
        return self._new("yaksa_type_create_hindexed_block", len(displs), bl, _arr(_ip, displs), old)

    def type_create_indexed(self, blens, displs, old):
        return self._new("yaksa_type_create_indexed", len(blens), _arr(_ip, blens), _arr(_ip, displs),
                         old)

    def type_create_hindexed(self, blens, displs, old):
        return self._new("yaksa_type_create_hindexed", len(blens), _arr(_ip, blens), _arr(_ip, displs),
                         old)

    def type_create_hindexed_arrays(self, count, blens_ptr, displs_ptr, old):
        """hindexed from raw intptr_t arrays (numpy .ctypes.data) for large counts."""
        return self._new("yaksa_type_create_hindexed", count, ctypes.cast(blens_ptr, ctypes.POINTER(_ip)),
                         ctypes.cast(displs_ptr, ctypes.POINTER(_ip)), old)

    def type_create_hindexed_block_array(self, count, bl, displs_ptr, old):
        return self._new("yaksa_type_create_hindexed_block", count, bl,
                         ctypes.cast(displs_ptr, ctypes.POINTER(_ip)), old)

    def type_create_indexed_block_array(self, count, bl, displs_ptr, old):
        return self._new("yaksa_type_create_indexed_block", count, bl,
                         ctypes.cast(displs_ptr, ctypes.POINTER(_ip)), old)

    def type_create_resized(self, old, lb, extent):
        return self._new("yaksa_type_create_resized", old, lb, extent)

    def type_create_struct(self, blens, displs, types):
        return self._new("yaksa_type_create_struct", len(blens), _arr(_ip, blens), _arr(_ip, displs),
                         _arr(_u64, types))

    def type_create_subarray(self, sizes, subsizes, starts, order, old):
        n = len(sizes)
        return self._new("yaksa_type_create_subarray", n, _arr(_ip, sizes), _arr(_ip, subsizes),
                         _arr(_ip, starts), order, old)

    def type_free(self, t):
        self._chk("yaksa_type_free", self.lib.yaksa_type_free(t))

    def size(self, t):
        s = _up()
        self._chk("yaksa_type_get_size", self.lib.yaksa_type_get_size(t, ctypes.byref(s)))
        return s.value

    def extent(self, t):
        lb, ext = _ip(), _ip()
        self._chk("yaksa_type_get_extent", self.lib.yaksa_type_get_extent(t, ctypes.byref(lb),
                                                                           ctypes.byref(ext)))
        return lb.value, ext.value

    def true_extent(self, t):
        lb, ext = _ip(), _ip()
        self._chk("yaksa_type_get_true_extent",
                  self.lib.yaksa_type_get_true_extent(t, ctypes.byref(lb), ctypes.byref(ext)))
        return lb.value, ext.value

    def iov_len(self, count, t):
        n = _up()
        self._chk("yaksa_iov_len", self.lib.yaksa_iov_len(count, t, ctypes.byref(n)))
        return n.value

    def iov_len_max(self, count, t, max_bytes):
        n, b = _up(), _up()
        self._chk("yaksa_iov_len_max", self.lib.yaksa_iov_len_max(count, t, max_bytes, ctypes.byref(n),
                                                                   ctypes.byref(b)))
        return n.value, b.value

    def iov(self, buf, count, t, offset, max_len):
        """yaksa_iov; returns a list of (address, length)."""
        arr = (IoVec * max(1, max_len))()
        n = _up()
        self._chk("yaksa_iov", self.lib.yaksa_iov(buf, count, t, offset, arr, max_len, ctypes.byref(n)))
        return [(arr[i].iov_base or 0, arr[i].iov_len) for i in range(n.value)]

    def flatten(self, t):
        """yaksa_flatten_size + yaksa_flatten; returns the bytes."""
        n = _up()
        self._chk("yaksa_flatten_size", self.lib.yaksa_flatten_size(t, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(max(1, n.value))
        self._chk("yaksa_flatten", self.lib.yaksa_flatten(t, buf))
        return buf.raw[:n.value]

    def unflatten(self, data):
        buf = ctypes.create_string_buffer(data, len(data))
        h = _u64()
        self._chk("yaksa_unflatten", self.lib.yaksa_unflatten(ctypes.byref(h), buf))
        return h.value

    # pack / unpack: pointers are plain integers (device or host addresses)
    def ipack(self, inbuf, incount, t, inoffset, outbuf, max_bytes, op=OP_REPLACE, info=None):
        actual, req = _up(), _u64()
        rc = self.lib.yaksa_ipack(inbuf, incount, t, inoffset, outbuf, max_bytes, ctypes.byref(actual),
                                  info, op, ctypes.byref(req))
        self._chk("yaksa_ipack", rc)
        return actual.value, req.value

    def iunpack(self, inbuf, insize, outbuf, outcount, t, outoffset, op=OP_REPLACE, info=None):
        actual, req = _up(), _u64()
        rc = self.lib.yaksa_iunpack(inbuf, insize, outbuf, outcount, t, outoffset, ctypes.byref(actual),
                                    info, op, ctypes.byref(req))
        self._chk("yaksa_iunpack", rc)
        return actual.value, req.value

    def pack(self, inbuf, incount, t, inoffset, outbuf, max_bytes, op=OP_REPLACE, info=None):
        actual = _up()
        self._chk("yaksa_pack", self.lib.yaksa_pack(inbuf, incount, t, inoffset, outbuf, max_bytes,
                                                    ctypes.byref(actual), info, op))
        return actual.value

    def unpack(self, inbuf, insize, outbuf, outcount, t, outoffset, op=OP_REPLACE, info=None):
        actual = _up()
        self._chk("yaksa_unpack", self.lib.yaksa_unpack(inbuf, insize, outbuf, outcount, t, outoffset,
                                                        ctypes.byref(actual), info, op))
        return actual.value

    def pack_stream(self, inbuf, incount, t, inoffset, outbuf, max_bytes, stream_ptr, op=OP_REPLACE,
                    info=None):
        """stream_ptr: address of a cudaStream_t (as the reference API expects)."""
        actual = _up()
        self._chk("yaksa_pack_stream", self.lib.yaksa_pack_stream(inbuf, incount, t, inoffset, outbuf,
                                                                  max_bytes, ctypes.byref(actual),
                                                                  info, op, stream_ptr))
        return actual.value

    def unpack_stream(self, inbuf, insize, outbuf, outcount, t, outoffset, stream_ptr, op=OP_REPLACE,
                      info=None):
        actual = _up()
        self._chk("yaksa_unpack_stream", self.lib.yaksa_unpack_stream(inbuf, insize, outbuf, outcount, t,
                                                                      outoffset, ctypes.byref(actual),
                                                                      info, op, stream_ptr))
        return actual.value

    def wait(self, req):
        self._chk("yaksa_request_wait", self.lib.yaksa_request_wait(req))

    def test(self, req):
        c = ctypes.c_int()
        self._chk("yaksa_request_test", self.lib.yaksa_request_test(req, ctypes.byref(c)))
        return bool(c.value)

    # batches (include/yaksa_gb300.h)
    @staticmethod
    def batch_array(ops):
        arr = (PupOp * len(ops))(*ops)
        return arr

    def pup_batch(self, arr, info=None):
        self._chk("yaksa_gb300_pup_batch", self.lib.yaksa_gb300_pup_batch(arr, len(arr), info))
        return [o.actual for o in arr]

    def pup_batch_stream(self, arr, stream_ptr, info=None):
        self._chk("yaksa_gb300_pup_batch_stream",
                  self.lib.yaksa_gb300_pup_batch_stream(arr, len(arr), info, stream_ptr))

    def ipup_batch(self, arr, info=None):
        req = _u64()
        self._chk("yaksa_gb300_ipup_batch",
                  self.lib.yaksa_gb300_ipup_batch(arr, len(arr), info, ctypes.byref(req)))
        return req.value

    def graph_create(self, batches, info=None):
        """batches: list of lists of PupOp; returns (graph handle, flat PupOp array)."""
        flat = [o for b in batches for o in b]
        arr = (PupOp * len(flat))(*flat)
        ends, acc = [], 0
        for b in batches:
            acc += len(b)
            ends.append(acc)
        e = (ctypes.c_int * len(ends))(*ends)
        g = _vp()
        self._chk("yaksa_gb300_graph_create",
                  self.lib.yaksa_gb300_graph_create(arr, e, len(ends), info, ctypes.byref(g)))
        return g, arr

    def pup_noalloc(self, op, stream_ptr=None):
        """yaksa_gb300_pup_noalloc: one request through the static descriptor scratch;
        returns the YAKSA_* code (0 on success) and sets op.actual."""
        return self.lib.yaksa_gb300_pup_noalloc(ctypes.byref(op), stream_ptr)

    def probe_rows(self, rows, write, stream_ptr=None):
        """yaksa_gb300_probe_rows: touch the runs of up to 16 Rows patterns in one launch
        (loads, or stores of zeros when `write`)."""
        arr = (Rows * len(rows))(*rows)
        self._chk("yaksa_gb300_probe_rows", self.lib.yaksa_gb300_probe_rows(arr, len(rows), int(write),
                                                                            stream_ptr))

    def graph_launch(self, g, stream_ptr=None):
        self._chk("yaksa_gb300_graph_launch", self.lib.yaksa_gb300_graph_launch(g, stream_ptr))

    def graph_free(self, g):
        self._chk("yaksa_gb300_graph_free", self.lib.yaksa_gb300_graph_free(g))

    def shard(self, t, count, rank, nranks):
        """yaksa_gb300_shard: (inoffset, bytes) of rank's part of the packed range."""
        o, n = _up(), _up()
        self._chk("yaksa_gb300_shard", self.lib.yaksa_gb300_shard(t, count, rank, nranks,
                                                                   ctypes.byref(o), ctypes.byref(n)))
        return o.value, n.value

    def graph_lane_stats(self):
        c, r = _u64(), _u64()
        self.lib.yaksa_gb300_graph_lane_stats(ctypes.byref(c), ctypes.byref(r))
        return dict(captures=c.value, replays=r.value)

    def autotune_stats(self):
        a, b, c = ctypes.c_uint32(), ctypes.c_uint32(), _u64()
        self.lib.yaksa_gb300_autotune_stats(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return dict(classes=a.value, decided=b.value, probes=c.value)

    def stats(self):
        v = [_u64() for _ in range(4)]
        self.lib.yaksa_gb300_stats(*[ctypes.byref(x) for x in v])
        return dict(zip(["launches", "direct_calls", "staged_calls", "memcpy_calls"],
                        [x.value for x in v]))
