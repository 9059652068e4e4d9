"""ctypes binding of the C ABI (include/iss_gpu.h) and a Python class with
the method names of the reference's driver class iSS (src/iSS.h:16-102).

There is no CPU path: every call runs through iss_gb300/_native/libiss_gb300.so
and the GPU kernels behind it; if the library is missing the import fails
with instructions to build it."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_native", "libiss_gb300.so")
TABLE_DIR = os.path.join(HERE, "data", "iSS_tables")

HADRON_DTYPE = np.dtype([("pid", "<i4"), ("mass", "<f4"), ("E", "<f4"), ("px", "<f4"),
                         ("py", "<f4"), ("pz", "<f4"), ("t", "<f4"), ("x", "<f4"),
                         ("y", "<f4"), ("z", "<f4")])

ISS_OK = 0
STATUS = {0: "ISS_OK", 1: "ISS_ERR_INVALID_ARG", 2: "ISS_ERR_IO", 3: "ISS_ERR_PARAM_MISSING",
          4: "ISS_ERR_UNSUPPORTED", 5: "ISS_ERR_CUDA", 6: "ISS_ERR_OUT_OF_RANGE",
          7: "ISS_ERR_NO_SURFACE", 8: "ISS_ERR_NO_SAMPLES", 9: "ISS_ERR_CAPACITY",
          10: "ISS_ERR_SAMPLING"}
OUTPUT_OSCAR, OUTPUT_GZIP, OUTPUT_BINARY = 1, 2, 3

EXPORTED = [
    "iss_gpu_create", "iss_gpu_destroy", "iss_gpu_set_param", "iss_gpu_get_param",
    "iss_gpu_parse_param_line", "iss_gpu_set_seed", "iss_gpu_set_seed_from_params",
    "iss_gpu_read_surface", "iss_gpu_set_surface", "iss_gpu_set_surface_batch",
    "iss_gpu_generate", "iss_gpu_generate_into", "iss_gpu_generate_stream",
    "iss_gpu_shell",
    "iss_gpu_clear", "iss_gpu_num_events", "iss_gpu_num_particles", "iss_gpu_get_hadron",
    "iss_gpu_copy_event", "iss_gpu_copy_all", "iss_gpu_write_output",
    "iss_gpu_write_hadron_list", "iss_gpu_species",
    "iss_gpu_species_yields", "iss_gpu_num_cells", "iss_gpu_copy_lrf_cells",
    "iss_gpu_copy_cell_yields", "iss_gpu_copy_counts", "iss_gpu_get_timings",
    "iss_gpu_last_error", "iss_gpu_status_string", "iss_gpu_scan_counts_noalloc",
    "iss_gpu_learned_num_weights", "iss_gpu_learned_init_weights", "iss_gpu_learned_set_weights",
    "iss_gpu_learned_get_weights", "iss_gpu_learned_forward", "iss_gpu_learned_loss_grad",
    "iss_gpu_mma_selftest", "iss_gpu_learned_train", "iss_gpu_learned_stats",
    "iss_gpu_learned_copy_rows", "iss_gpu_get_tuning", "iss_gpu_set_tuning", "iss_gpu_autotune",
]


# iss_stream_fn(user, hadrons, n_hadrons, first_event, n_events, event_offsets)
STREAM_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32,
                        C.POINTER(C.c_int64))


class Timings(C.Structure):
    _fields_ = [("ms_prologue", C.c_double), ("ms_yields", C.c_double), ("ms_cdf", C.c_double),
                ("ms_counts", C.c_double), ("ms_sample", C.c_double), ("ms_total", C.c_double),
                ("n_hadrons", C.c_int64), ("n_tries", C.c_int64),
                ("n_cell_redraws", C.c_int64), ("n_failures", C.c_int64),
                ("kernel_launches", C.c_int32), ("ms_decays", C.c_double),
                ("decay_reruns", C.c_int32), ("n_sampled", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class LearnedTrain(C.Structure):
    _fields_ = [("n_momenta", C.c_int64), ("first_seed", C.c_int32), ("n_seeds", C.c_int32),
                ("n_steps", C.c_int32), ("batch", C.c_int32), ("learning_rate", C.c_double),
                ("init_seed", C.c_uint64)]


class LearnedStats(C.Structure):
    _fields_ = [("n_species", C.c_int32), ("n_pairs", C.c_int64), ("ms_network", C.c_double),
                ("n_tries", C.c_int64), ("n_hadrons", C.c_int64), ("n_violations", C.c_int64),
                ("n_train_rows", C.c_int64), ("ms_train", C.c_double),
                ("train_events_per_seed", C.c_int32), ("train_nll_plain", C.c_double),
                ("ms_forward", C.c_double), ("n_excess_tries", C.c_int64),
                ("n_excess_hadrons", C.c_int64), ("n_over_one", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tuning(C.Structure):
    _fields_ = [("item_size", C.c_int32), ("yield_groups", C.c_int32), ("sampler_ctas", C.c_int32),
                ("assign_blocks", C.c_int32), ("copy_chunks", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class IssError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


_lib = None


def lib():
    """The loaded native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with "
                              "`python -c 'import __graft_entry__ as g; g.build()'` "
                              "or `python iss_gb300/build.py`")
        L = C.CDLL(LIB_PATH)
        v, h = C.c_void_p, C.c_void_p
        L.iss_gpu_create.argtypes = [C.c_char_p] * 5 + [C.POINTER(C.c_void_p)]
        L.iss_gpu_destroy.argtypes = [h]
        L.iss_gpu_set_param.argtypes = [h, C.c_char_p, C.c_double]
        L.iss_gpu_get_param.argtypes = [h, C.c_char_p, C.POINTER(C.c_double)]
        L.iss_gpu_parse_param_line.argtypes = [h, C.c_char_p]
        L.iss_gpu_set_seed.argtypes = [h, C.c_int64]
        L.iss_gpu_set_seed_from_params.argtypes = [h]
        L.iss_gpu_read_surface.argtypes = [h]
        L.iss_gpu_set_surface.argtypes = [h, v, C.c_int64]
        L.iss_gpu_set_surface_batch.argtypes = [h, v, v, v, C.c_int32]
        L.iss_gpu_generate.argtypes = [h]
        L.iss_gpu_generate_into.argtypes = [h, v, C.c_int64, C.POINTER(C.c_int64)]
        L.iss_gpu_generate_stream.argtypes = [h, C.c_int32, STREAM_FN, v]
        L.iss_gpu_shell.argtypes = [h]
        L.iss_gpu_clear.argtypes = [h]
        L.iss_gpu_num_events.argtypes = [h, C.POINTER(C.c_int32)]
        L.iss_gpu_num_particles.argtypes = [h, C.c_int32, C.POINTER(C.c_int64)]
        L.iss_gpu_get_hadron.argtypes = [h, C.c_int32, C.c_int64, v]
        L.iss_gpu_copy_event.argtypes = [h, C.c_int32, v, C.c_int64, C.POINTER(C.c_int64)]
        L.iss_gpu_copy_all.argtypes = [h, v, C.c_int64, v, C.POINTER(C.c_int64)]
        L.iss_gpu_write_output.argtypes = [h, C.c_int, C.c_char_p]
        L.iss_gpu_write_hadron_list.argtypes = [C.c_int, C.c_char_p, C.c_char_p, v, v, C.c_int32]
        L.iss_gpu_species.argtypes = [h, C.POINTER(C.c_int32), v, C.c_int32]
        L.iss_gpu_species_yields.argtypes = [h, v, C.c_int32]
        L.iss_gpu_num_cells.argtypes = [h, C.POINTER(C.c_int64)]
        L.iss_gpu_copy_lrf_cells.argtypes = [h, v, C.c_int64]
        L.iss_gpu_copy_cell_yields.argtypes = [h, C.c_int32, v, C.c_int64]
        L.iss_gpu_copy_counts.argtypes = [h, v, C.c_int64]
        L.iss_gpu_get_timings.argtypes = [h, C.POINTER(Timings)]
        L.iss_gpu_last_error.argtypes = [h]
        L.iss_gpu_last_error.restype = C.c_char_p
        L.iss_gpu_status_string.argtypes = [C.c_int]
        L.iss_gpu_status_string.restype = C.c_char_p
        L.iss_gpu_scan_counts_noalloc.argtypes = [v, C.c_int64, v, v]
        L.iss_gpu_learned_num_weights.argtypes = []
        L.iss_gpu_learned_init_weights.argtypes = [h, C.c_uint64]
        L.iss_gpu_learned_set_weights.argtypes = [h, v, C.c_int64]
        L.iss_gpu_learned_get_weights.argtypes = [h, v, C.c_int64]
        L.iss_gpu_learned_forward.argtypes = [h, v, C.c_int64, v]
        L.iss_gpu_learned_loss_grad.argtypes = [h, v, v, C.c_int64, C.POINTER(C.c_double), v]
        L.iss_gpu_mma_selftest.argtypes = [v, v, C.c_int32, C.c_int32, v]
        L.iss_gpu_learned_train.argtypes = [h, C.POINTER(LearnedTrain), v, C.c_int32]
        L.iss_gpu_learned_stats.argtypes = [h, C.POINTER(LearnedStats)]
        L.iss_gpu_learned_copy_rows.argtypes = [h, C.c_int64, C.c_int64, v, v]
        L.iss_gpu_get_tuning.argtypes = [h, C.POINTER(Tuning)]
        L.iss_gpu_set_tuning.argtypes = [h, C.POINTER(Tuning)]
        L.iss_gpu_autotune.argtypes = [h, C.POINTER(Tuning), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]
        for name in EXPORTED:
            if name not in ("iss_gpu_last_error", "iss_gpu_status_string"):
                getattr(L, name).restype = C.c_int
        L.iss_gpu_learned_num_weights.restype = C.c_int64
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class iSS:
    """The reference's iSS driver (src/iSS.h), GPU-backed.

    iSS(path, table_path, particle_table_path, inputfile, surface_filename)
    reads `inputfile` with ParameterReader rules; table paths default to the
    tables shipped in iss_gb300/data."""

    def __init__(self, path=".", table_path=TABLE_DIR, particle_table_path=None,
                 inputfile="", surface_filename="surface.dat"):
        self._L = lib()
        h = C.c_void_p()
        pt = particle_table_path or table_path
        st = self._L.iss_gpu_create(path.encode(), table_path.encode(), pt.encode(),
                                    inputfile.encode(), surface_filename.encode(), C.byref(h))
        if st != ISS_OK:
            raise IssError(st, f"can not create sampler (parameter file {inputfile!r})")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.iss_gpu_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st):
        if st != ISS_OK:
            raise IssError(st, self._L.iss_gpu_last_error(self._h).decode())
        return st

    # ParameterReader
    def setVal(self, key, value):
        self._check(self._L.iss_gpu_set_param(self._h, key.encode(), float(value)))

    def getVal(self, key, default=None):
        v = C.c_double()
        st = self._L.iss_gpu_get_param(self._h, key.encode(), C.byref(v))
        if st != ISS_OK:
            if default is not None:
                return default
            self._check(st)
        return v.value

    def readFromArguments(self, args):
        for a in args:
            self._check(self._L.iss_gpu_parse_param_line(self._h, a.encode()))

    def set_params(self, **kw):
        for k, v in kw.items():
            self.setVal(k, v)

    # iSS
    def set_random_seed(self, seed=None):
        if seed is None:
            self._check(self._L.iss_gpu_set_seed_from_params(self._h))
        else:
            self._check(self._L.iss_gpu_set_seed(self._h, int(seed)))

    def read_in_FO_surface(self):
        return self._check(self._L.iss_gpu_read_surface(self._h))

    def set_surface(self, fo_surf_records):
        a = np.ascontiguousarray(fo_surf_records, dtype=np.float32)
        assert a.ndim == 2 and a.shape[1] == 34
        self._check(self._L.iss_gpu_set_surface(self._h, _ptr(a), a.shape[0]))

    def set_surface_batch(self, surfaces, events):
        """Several FO_surf record arrays, sampled together by one
        generate_samples; events[b] events for surface b, numbered across the
        batch in surface order."""
        recs = np.ascontiguousarray(np.concatenate([np.asarray(r, dtype=np.float32)
                                                    for r in surfaces]), dtype=np.float32)
        off = np.zeros(len(surfaces) + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(r) for r in surfaces])
        ev = np.ascontiguousarray(events, dtype=np.int32)
        return self._check(self._L.iss_gpu_set_surface_batch(self._h, _ptr(recs), _ptr(off),
                                                             _ptr(ev), len(surfaces)))

    def set_surface_batch_flat(self, records, cell_offsets, events):
        """set_surface_batch on records already concatenated (float32 [n][34],
        e.g. page-locked) with cell_offsets[b] the first record of surface b
        (n_surfaces + 1 entries): no host copy before the C ABI call."""
        assert records.dtype == np.float32 and records.flags.c_contiguous and records.shape[1] == 34
        off = np.ascontiguousarray(cell_offsets, dtype=np.int64)
        ev = np.ascontiguousarray(events, dtype=np.int32)
        return self._check(self._L.iss_gpu_set_surface_batch(self._h, _ptr(records), _ptr(off),
                                                             _ptr(ev), len(ev)))

    def generate_samples(self):
        return self._check(self._L.iss_gpu_generate(self._h))

    def generate_into(self, out):
        """generate_samples with every event's hadrons copied into `out` (a
        HADRON_DTYPE array, best in pinned memory) while later events are
        still being sampled; returns (hadrons, event_offsets)."""
        n = C.c_int64()
        self._check(self._L.iss_gpu_generate_into(self._h, _ptr(out), out.size, C.byref(n)))
        nev = self.get_number_of_sampled_events()
        off = np.zeros(nev + 1, dtype=np.int64)
        self._check(self._L.iss_gpu_copy_all(self._h, None, 0, _ptr(off), None))
        return out[:n.value], off

    def generate_stream(self, chunk_events, fn):
        """generate_samples with the hadrons handed to fn(hadrons, first_event,
        event_offsets) chunk by chunk (chunk_events events each) instead of
        kept: `hadrons` is a HADRON_DTYPE view of the library's page-locked
        buffer, valid only during the call (copy what you keep); event k of
        the chunk is hadrons[event_offsets[k]:event_offsets[k+1]].  The device
        holds two chunks of records at a time."""
        errors = []

        def tramp(user, ptr, n, first, nev, off):
            try:
                offs = np.ctypeslib.as_array(off, shape=(nev + 1,)).copy()
                if n > 0:
                    buf = (C.c_char * (int(n) * HADRON_DTYPE.itemsize)).from_address(ptr)
                    had = np.frombuffer(buf, dtype=HADRON_DTYPE, count=int(n))
                else:
                    had = np.zeros(0, dtype=HADRON_DTYPE)
                fn(had, int(first), offs)
            except Exception as e:   # re-raised after the call
                errors.append(e)

        cb = STREAM_FN(tramp)
        st = self._L.iss_gpu_generate_stream(self._h, int(chunk_events), cb, None)
        if errors:
            raise errors[0]
        return self._check(st)

    def shell(self):
        return self._check(self._L.iss_gpu_shell(self._h))

    def clear(self):
        self._check(self._L.iss_gpu_clear(self._h))

    def get_number_of_sampled_events(self):
        n = C.c_int32()
        self._check(self._L.iss_gpu_num_events(self._h, C.byref(n)))
        return n.value

    def get_number_of_particles(self, iev):
        n = C.c_int64()
        self._check(self._L.iss_gpu_num_particles(self._h, iev, C.byref(n)))
        return n.value

    def get_hadron(self, iev, ipart):
        out = np.zeros(1, dtype=HADRON_DTYPE)
        self._check(self._L.iss_gpu_get_hadron(self._h, iev, ipart, _ptr(out)))
        return out[0]

    def get_hadron_list_iev(self, iev):
        n = C.c_int64()
        self._check(self._L.iss_gpu_copy_event(self._h, iev, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=HADRON_DTYPE)
        if n.value:
            self._check(self._L.iss_gpu_copy_event(self._h, iev, _ptr(out), n.value, C.byref(n)))
        return out

    def event_offsets(self):
        """First hadron of every event (n_events + 1 entries), without copying hadrons."""
        nev = self.get_number_of_sampled_events()
        off = np.zeros(nev + 1, dtype=np.int64)
        n = C.c_int64()
        self._check(self._L.iss_gpu_copy_all(self._h, None, 0, _ptr(off), C.byref(n)))
        return off

    def all_hadrons(self, out=None):
        """(hadrons, event_offsets): every event in one device->host copy."""
        n = C.c_int64()
        nev = self.get_number_of_sampled_events()
        off = np.zeros(nev + 1, dtype=np.int64)
        self._check(self._L.iss_gpu_copy_all(self._h, None, 0, _ptr(off), C.byref(n)))
        if out is None or out.size < n.value:
            out = np.zeros(n.value, dtype=HADRON_DTYPE)
        if n.value:
            self._check(self._L.iss_gpu_copy_all(self._h, _ptr(out), out.size, None, C.byref(n)))
        return out[:n.value], off

    def write_output(self, fmt, filename=None):
        self._check(self._L.iss_gpu_write_output(self._h, fmt,
                                                 filename.encode() if filename else None))

    # inspection
    def species(self):
        n = C.c_int32()
        self._check(self._L.iss_gpu_species(self._h, C.byref(n), None, 0))
        out = np.zeros(n.value, dtype=np.int32)
        self._check(self._L.iss_gpu_species(self._h, C.byref(n), _ptr(out), n.value))
        return out

    def species_yields(self):
        n = len(self.species())
        out = np.zeros(n, dtype=np.float64)
        self._check(self._L.iss_gpu_species_yields(self._h, _ptr(out), n))
        return out

    def num_cells(self):
        n = C.c_int64()
        self._check(self._L.iss_gpu_num_cells(self._h, C.byref(n)))
        return n.value

    def lrf_cells(self):
        n = self.num_cells()
        out = np.zeros((n, 28), dtype=np.float32)
        self._check(self._L.iss_gpu_copy_lrf_cells(self._h, _ptr(out), n))
        return out

    def cell_yields(self, species_index=None):
        n = self.num_cells()
        if species_index is not None:
            out = np.zeros(n, dtype=np.float32)
            self._check(self._L.iss_gpu_copy_cell_yields(self._h, species_index, _ptr(out), n))
            return out
        ns = len(self.species())
        out = np.zeros((ns, n), dtype=np.float32)
        for k in range(ns):
            self._check(self._L.iss_gpu_copy_cell_yields(self._h, k, _ptr(out[k]), n))
        return out

    def counts(self):
        nev = self.get_number_of_sampled_events()
        ns = len(self.species())
        out = np.zeros((nev, ns), dtype=np.int32)
        self._check(self._L.iss_gpu_copy_counts(self._h, _ptr(out), out.size))
        return out

    def timings(self):
        t = Timings()
        self._check(self._L.iss_gpu_get_timings(self._h, C.byref(t)))
        return t.as_dict()

    # launch shape
    def get_tuning(self):
        t = Tuning()
        self._check(self._L.iss_gpu_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, **kw):
        t = Tuning(**dict(self.get_tuning(), **kw))
        self._check(self._L.iss_gpu_set_tuning(self._h, C.byref(t)))

    def autotune(self):
        """Tunes the launch shape on this handle's workload; returns (shape,
        ms before, ms after)."""
        t = Tuning()
        b, a = C.c_double(), C.c_double()
        self._check(self._L.iss_gpu_autotune(self._h, C.byref(t), C.byref(b), C.byref(a)))
        return t.as_dict(), b.value, a.value

    # the learned proposal network
    def learned_init_weights(self, seed=0):
        self._check(self._L.iss_gpu_learned_init_weights(self._h, int(seed)))

    def learned_set_weights(self, w):
        a = np.ascontiguousarray(w, dtype=np.float32)
        self._check(self._L.iss_gpu_learned_set_weights(self._h, _ptr(a), a.size))

    def learned_get_weights(self):
        out = np.zeros(self._L.iss_gpu_learned_num_weights(), dtype=np.float32)
        self._check(self._L.iss_gpu_learned_get_weights(self._h, _ptr(out), out.size))
        return out

    def learned_forward(self, features):
        f = np.ascontiguousarray(features, dtype=np.float32)
        out = np.zeros((f.shape[0], 64), dtype=np.float32)
        self._check(self._L.iss_gpu_learned_forward(self._h, _ptr(f), f.shape[0], _ptr(out)))
        return out

    def learned_loss_grad(self, features, targets):
        f = np.ascontiguousarray(features, dtype=np.float32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        g = np.zeros(self._L.iss_gpu_learned_num_weights(), dtype=np.float32)
        loss = C.c_double()
        self._check(self._L.iss_gpu_learned_loss_grad(self._h, _ptr(f), _ptr(t), f.shape[0],
                                                      C.byref(loss), _ptr(g)))
        return loss.value, g


    def learned_train(self, n_momenta=50_000_000, first_seed=10, n_seeds=10, n_steps=2000,
                      batch=8192, learning_rate=1e-3, init_seed=0):
        """Train the proposal network on momenta of the plain sampler; returns
        the mean loss of every step."""
        o = LearnedTrain(int(n_momenta), int(first_seed), int(n_seeds), int(n_steps), int(batch),
                         float(learning_rate), int(init_seed))
        curve = np.zeros(max(int(n_steps), 1), dtype=np.float64)
        self._check(self._L.iss_gpu_learned_train(self._h, C.byref(o), _ptr(curve), curve.size))
        return curve[:int(n_steps)]

    def learned_stats(self):
        st = LearnedStats()
        self._check(self._L.iss_gpu_learned_stats(self._h, C.byref(st)))
        return st.as_dict()

    def learned_rows(self, first, count):
        f = np.zeros((count, 18), dtype=np.float32)
        t = np.zeros((count, 4), dtype=np.float32)
        self._check(self._L.iss_gpu_learned_copy_rows(self._h, int(first), int(count), _ptr(f), _ptr(t)))
        return f, t


def mma_selftest(a_bf16, b_bf16):
    """c = a @ b.T on one tensor-core tile (a: [128][k], b: [n][k], raw bf16
    bit patterns as uint16)."""
    a = np.ascontiguousarray(a_bf16, dtype=np.uint16)
    b = np.ascontiguousarray(b_bf16, dtype=np.uint16)
    c = np.zeros((128, b.shape[0]), dtype=np.float32)
    st = lib().iss_gpu_mma_selftest(_ptr(a), _ptr(b), b.shape[0], a.shape[1], _ptr(c))
    if st != ISS_OK:
        raise IssError(st, "tensor-core self-test failed")
    return c


def write_hadron_list(fmt, filename, hadrons, event_offsets, table_path=TABLE_DIR):
    """The reference's output writers (OSCAR / gzip / binary) on a host hadron
    list: events [event_offsets[i], event_offsets[i+1]) of `hadrons`
    (HADRON_DTYPE).  No device is needed."""
    h = np.ascontiguousarray(hadrons, dtype=HADRON_DTYPE)
    off = np.ascontiguousarray(event_offsets, dtype=np.int64)
    st = lib().iss_gpu_write_hadron_list(int(fmt), filename.encode(),
                                         table_path.encode() if table_path else None,
                                         _ptr(h) if h.size else None, _ptr(off), len(off) - 1)
    if st != ISS_OK:
        raise IssError(st, f"iss_gpu_write_hadron_list({fmt}, {filename})")
