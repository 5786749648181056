"""Many scenes through one persistent forward launch (tp_batch_* in include/tp.h)."""
import ctypes as C

from . import _lib as L


class Batch:
    def __init__(self, processors):
        self._lib = L.load()
        self.processors = list(processors)  # kept alive: the batch borrows their device buffers
        arr = (C.c_void_p * len(self.processors))(*[p.h for p in self.processors])
        self.h = C.c_void_p()
        st = self._lib.tp_batch_create(arr, len(self.processors), C.byref(self.h))
        if st != L.TP_OK:
            raise L.TpError(st, "tp_batch_create")

    def _ck(self, st, what):
        if st != L.TP_OK:
            buf = C.create_string_buffer(512)
            self._lib.tp_batch_last_error(self.h, buf, 512)
            raise L.TpError(st, "%s: %s" % (what, buf.value.decode(errors="replace")))

    def process(self, replan=True, stream=None):
        self._ck(self._lib.tp_batch_process(self.h, int(bool(replan)), stream), "tp_batch_process")

    def run_graph(self, stream=None):
        self._ck(self._lib.tp_batch_run_graph(self.h, stream), "tp_batch_run_graph")

    def synchronize(self):
        self._ck(self._lib.tp_batch_synchronize(self.h), "tp_batch_synchronize")

    def close(self):
        if getattr(self, "h", None):
            self._lib.tp_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
