"""CPU decode of CPHD signal arrays -- TEST INFRASTRUCTURE ONLY (the checker for
sarsolver_gb300.cphd and sar_cphd_decode; the product never imports it).

Restates the published CPHD sample formats (CPHD 1.0.1 Data/SignalArrayFormat CI2 / CI4 / CF8;
CPHD 0.3 Data/SampleType RE08I_IM08I / RE16I_IM16I / RE32F_IM32F): big-endian interleaved (I, Q)
pairs of signed 8-bit or 16-bit integers or IEEE binary32, scaled per vector by the AmpSF
parameter when present.  The reference decodes through sarpy (src/sarsolver/io/cphd101.py:251-265,
io/cphd03.py:250-263), which is not installed here, and its only file test downloads a public
collection over the network (tests/conftest.py:16-34), so no reference-produced file or output
exists: parity unpinned against sarpy.  Two independent restatements are given (numpy big-endian
types, and byte-by-byte with struct), and they are checked against each other.
"""
from __future__ import annotations

import struct
from typing import Optional

import numpy as np

_NP = {"CI2": ">i1", "CI4": ">i2", "CF8": ">f4"}
_STRUCT = {"CI2": (">b", 1), "CI4": (">h", 2), "CF8": (">f", 4)}


def decode_signal(raw, fmt: str, num_vectors: int, num_samples: int, amp_sf: Optional[np.ndarray] = None) -> np.ndarray:
    """complex64 [num_vectors, num_samples]: float32(I) + i float32(Q), times float32(AmpSF[v])."""
    comp = np.frombuffer(np.asarray(raw, dtype=np.uint8).tobytes(), dtype=_NP[fmt]).astype(np.float32)
    comp = comp.reshape(num_vectors, num_samples, 2)
    if amp_sf is not None:
        comp = comp * np.asarray(amp_sf, dtype=np.float32)[:, None, None]   # float32 products
    out = np.empty((num_vectors, num_samples), dtype=np.complex64)
    out.real, out.imag = comp[..., 0], comp[..., 1]
    return out


def decode_signal_bytewise(raw: bytes, fmt: str, num_vectors: int, num_samples: int,
                           amp_sf: Optional[np.ndarray] = None) -> np.ndarray:
    """The same, one component at a time through struct (small cases only)."""
    code, size = _STRUCT[fmt]
    out = np.empty((num_vectors, num_samples), dtype=np.complex64)
    for v in range(num_vectors):
        a = np.float32(1.0) if amp_sf is None else np.float32(amp_sf[v])
        for s in range(num_samples):
            at = (v * num_samples + s) * 2 * size
            i = np.float32(struct.unpack(code, raw[at:at + size])[0])
            q = np.float32(struct.unpack(code, raw[at + size:at + 2 * size])[0])
            out[v, s] = np.complex64(complex(np.float32(i * a), np.float32(q * a)))
    return out
