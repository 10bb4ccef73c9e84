"""CPU oracle for the LSD radix-sort pass -- TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s cpu_baseline
leg (and its ``--impl reference`` arm) import this package; it is the checker,
never the thing measured as the product. It wraps, through ctypes:

* ``oracle/_build/liblsb_oracle.so`` -- the C restatement of
  mpi/mpi_lsbsort.cpp (mppf/distributed-lsb) at R simulated ranks;
* ``oracle/_ref/liblsb_ref.so`` -- the reference's own ``mySort`` and
  ``globalShuffle`` compiled from its source file, present only where the
  reference checkout was available when ``make -C oracle ref`` ran.

Arrays are numpy ``uint64`` arrays of shape (n, 2): column 0 the key, column 1
the value, the byte layout of the reference's ``SortElement``
(mpi/mpi_lsbsort.cpp:30-33).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liblsb_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "liblsb_ref.so")
REF_MAIN = os.path.join(HERE, "_ref", "mpi_lsbsort")
# The reference checkout: LSB_REFERENCE_DIR when set, otherwise a checkout
# named `reference` next to this repository (absent on machines that only run
# the prebuilt checker).
REFERENCE_DIR = os.environ.get("LSB_REFERENCE_DIR") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")
REFERENCE_SRC = os.path.join(REFERENCE_DIR, "mpi", "mpi_lsbsort.cpp")

DIST_UNIFORM, DIST_LOW32, DIST_ZIPF, DIST_EQUAL, DIST_NEARLY_SORTED = 0, 1, 2, 3, 4
DIST_NAMES = {"uniform": 0, "low32": 1, "zipf": 2, "equal": 3, "nearly_sorted": 4}
ZIPF_KEYS = 1 << 20
ZIPF_S = 1.1

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_lib = None
_ref = None
_zipf_cache: dict = {}


def build(with_ref: bool | None = None) -> None:
    """Compile the oracle (always) and the reference (when its source exists)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if with_ref is None:
        with_ref = os.path.exists(REFERENCE_SRC)
    if with_ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REFERENCE_DIR}"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(with_ref=False)
        L = ctypes.CDLL(ORACLE_SO)
        L.oracle_splitmix64.restype = ctypes.c_uint64
        L.oracle_splitmix64.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.oracle_zipf_thresholds.restype = None
        L.oracle_zipf_thresholds.argtypes = [_I64, ctypes.c_double, _P]
        L.oracle_generate.argtypes = [_P, _I64, ctypes.c_int, ctypes.c_uint64, _P]
        L.oracle_num_passes.argtypes = [ctypes.c_int]
        L.oracle_global_shuffle.argtypes = [_P, _P, _I64, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_mysort.argtypes = [_P, _P, _I64, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_histogram.argtypes = [_P, _I64, ctypes.c_int, _P]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        R = ctypes.CDLL(REF_SO)
        R.lsb_ref_mysort.argtypes = [_P, _I64]
        R.lsb_ref_global_shuffle.argtypes = [_P, _I64, ctypes.c_int]
        _ref = R
    return _ref


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P) if a.size else None


def zipf_thresholds(m: int = ZIPF_KEYS, s: float = ZIPF_S) -> np.ndarray:
    key = (m, s)
    if key not in _zipf_cache:
        t = np.empty(m, dtype=np.uint64)
        lib().oracle_zipf_thresholds(m, s, _ptr(t))
        _zipf_cache[key] = t
    return _zipf_cache[key]


def generate(n: int, dist: int = DIST_UNIFORM, seed: int = 1) -> np.ndarray:
    out = np.empty((n, 2), dtype=np.uint64)
    thr = zipf_thresholds() if dist == DIST_ZIPF else None
    rc = lib().oracle_generate(_ptr(out), n, dist, seed, _ptr(thr) if thr is not None else None)
    if rc != 0:
        raise ValueError(f"oracle_generate failed ({rc})")
    return out


def num_passes(digit_bits: int) -> int:
    return (64 + digit_bits - 1) // digit_bits


def mysort(a: np.ndarray, digit_bits: int = 16, ranks: int = 1, threads: int = 1) -> np.ndarray:
    """The reference's mySort restated: returns a sorted copy of `a`."""
    A = np.ascontiguousarray(a, dtype=np.uint64).copy()
    B = np.empty_like(A)
    rc = lib().oracle_mysort(_ptr(A), _ptr(B), A.shape[0], digit_bits, ranks, threads)
    if rc != 0:
        raise RuntimeError(f"oracle_mysort failed ({rc})")
    return A


def global_shuffle(a: np.ndarray, digit: int, digit_bits: int = 16, ranks: int = 1) -> np.ndarray:
    """One pass, the reference's globalShuffle restated: returns a new array."""
    A = np.ascontiguousarray(a, dtype=np.uint64).copy()
    B = np.empty_like(A)
    rc = lib().oracle_global_shuffle(_ptr(A), _ptr(B), A.shape[0], digit_bits, digit, ranks)
    if rc != 0:
        raise RuntimeError(f"oracle_global_shuffle failed ({rc})")
    return A


def histogram(a: np.ndarray, digit_bits: int = 16) -> np.ndarray:
    p = num_passes(digit_bits)
    counts = np.zeros((p, 1 << digit_bits), dtype=np.int64)
    A = np.ascontiguousarray(a, dtype=np.uint64)
    rc = lib().oracle_histogram(_ptr(A), A.shape[0], digit_bits, _ptr(counts))
    if rc != 0:
        raise RuntimeError(f"oracle_histogram failed ({rc})")
    return counts


def stable_sort_by_key(a: np.ndarray) -> np.ndarray:
    """The reference's known-answer check, std::stable_sort by key
    (mpi/mpi_lsbsort.cpp:766-771)."""
    order = np.argsort(a[:, 0], kind="stable")
    return a[order]


def ref_mysort(a: np.ndarray) -> np.ndarray:
    A = np.ascontiguousarray(a, dtype=np.uint64).copy()
    if ref().lsb_ref_mysort(_ptr(A), A.shape[0]) != 0:
        raise RuntimeError("lsb_ref_mysort failed")
    return A


def ref_global_shuffle(a: np.ndarray, digit: int) -> np.ndarray:
    A = np.ascontiguousarray(a, dtype=np.uint64).copy()
    if ref().lsb_ref_global_shuffle(_ptr(A), A.shape[0], digit) != 0:
        raise RuntimeError("lsb_ref_global_shuffle failed")
    return A
