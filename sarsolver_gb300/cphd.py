"""CPHD phase-history files, decoded on the GPU.

Drop-in counterparts of the reference's
  * ``io.Cphd101Dataset`` (src/sarsolver/io/cphd101.py:13-285) -> ``Cphd101Dataset``
  * ``io.Cphd03Dataset``  (src/sarsolver/io/cphd03.py:13-289)  -> ``Cphd03Dataset``
with the same constructor arguments, properties and methods.  The reference opens files through
sarpy's ``open_phase_history`` and decodes the signal arrays on the host; sarpy is not a dependency
here.  ``CphdReader`` parses the published file layouts itself and offers the two sarpy calls the
reference makes (``read_pvp_variable`` and ``read``):

  CPHD 1.0.x  header "CPHD/1.0.1", then ``KEY := value`` lines up to a form feed + newline;
              XML_BLOCK_*, PVP_BLOCK_*, SIGNAL_BLOCK_* give each block's size and byte offset.
              XML Data/SignalArrayFormat (CI2, CI4, CF8), Data/NumBytesPVP, Data/Channel
              (NumVectors, NumSamples, SignalArrayByteOffset, PVPArrayByteOffset), PVP/<name>
              (Offset and Size in 8-byte words, Format such as F8 or X=F8;Y=F8;Z=F8;), Global/SGN.
  CPHD 0.3    header "CPHD/0.3" with XML_DATA_*, XML_BYTE_OFFSET, VB_DATA_SIZE, VB_BYTE_OFFSET,
              CPHD_DATA_SIZE, CPHD_BYTE_OFFSET; Data/SampleType (RE08I_IM08I, RE16I_IM16I,
              RE32F_IM32F), Data/NumBytesVBP, Data/ArraySize per channel; VectorParameters lists
              each per-vector field's size in bytes in record order (FxParameters and
              TOAParameters nested); Global/PhaseSGN.  Channels follow one another in both blocks.

All binary values are big-endian.  Signal arrays go to the device as they lie in the file (2, 4 or
8 bytes per sample instead of complex64's 8) through two pinned host buffers filled by parallel
``preadv`` calls, and are widened there by ``sar_cphd_decode`` (times the per-vector AmpSF when the
file has one).  Per-vector parameters are small and read on the host.

``write_cphd`` writes the subset of either layout that this reader needs (a minimal file, not a
schema-complete one): simulated collections and test fixtures.
"""
from __future__ import annotations

import ctypes
import os
import threading
import xml.etree.ElementTree as ET
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _lib
from .geometry import C, NumpySimpleSarAperture, NumpySimpleSarDataset

SECTION_END = b"\x0c\n"
# signal format -> (sar_cphd_decode code, bytes per complex sample, big-endian component type)
FORMATS = {"CI2": (_lib.SAR_CPHD_CI2, 2, ">i1"), "CI4": (_lib.SAR_CPHD_CI4, 4, ">i2"), "CF8": (_lib.SAR_CPHD_CF8, 8, ">f4")}
SAMPLE_TYPES_03 = {"RE08I_IM08I": "CI2", "RE16I_IM16I": "CI4", "RE32F_IM32F": "CF8"}
_PVP_TYPES = {"F8": ">f8", "I8": ">i8", "U8": ">u8"}


@dataclass
class CphdChannel:
    identifier: str
    num_vectors: int
    num_samples: int
    signal_offset: int   # file offset of the channel's signal array
    pvp_offset: int      # file offset of the channel's per-vector parameter array


@dataclass
class PvpField:
    name: str
    byte_offset: int     # within one vector's record
    count: int           # values per vector
    dtype: Optional[str]  # big-endian numpy type, None when the format is not a plain 8-byte number


def _strip_namespaces(root: ET.Element) -> ET.Element:
    for el in root.iter():
        if isinstance(el.tag, str) and "}" in el.tag:
            el.tag = el.tag.split("}", 1)[1]
    return root


def _text(root: ET.Element, path: str, default=None) -> Optional[str]:
    el = root.find(path)
    return default if el is None or el.text is None else el.text.strip()


def _int(root: ET.Element, path: str) -> int:
    t = _text(root, path)
    if t is None:
        raise ValueError(f"CPHD XML has no {path}")
    return int(t)


def read_header(f) -> (str, Dict[str, str]):
    """(version, {key: value}) of the file header at the start of ``f``."""
    f.seek(0)
    head = f.read(1 << 16)
    end = head.find(SECTION_END)
    if not head.startswith(b"CPHD/") or end < 0:
        raise ValueError("not a CPHD file (no CPHD/<version> header ending in a form feed)")
    lines = head[:end].decode("ascii").splitlines()
    version = lines[0][len("CPHD/"):].strip()
    keys = {}
    for line in lines[1:]:
        if ":=" in line:
            k, v = line.split(":=", 1)
            keys[k.strip()] = v.strip()
    return version, keys


def _parse_pvp_format(fmt: str, size_words: int) -> (int, Optional[str]):
    """(count, dtype) of a CPHD 1.0 PVP Format string: a type code, or NAME=TYPE; pairs."""
    fmt = fmt.strip()
    parts = [p for p in fmt.split(";") if p.strip()]
    types = [p.split("=", 1)[1].strip() if "=" in p else p.strip() for p in parts]
    if types and all(t == types[0] for t in types) and types[0] in _PVP_TYPES and len(types) == size_words:
        return len(types), _PVP_TYPES[types[0]]
    return size_words, None


class CphdReader:
    """The parts of a CPHD file the operator needs (see the module docstring for the layouts)."""

    def __init__(self, path: str):
        self.path = os.fspath(path)
        with open(self.path, "rb") as f:
            self.version, self.header = read_header(f)
            if self.version.startswith("1."):
                self._parse_v1(f)
            elif self.version.startswith("0.3"):
                self._parse_v03(f)
            else:
                raise ValueError(f"unsupported CPHD version {self.version}")
        self._pvp_cache: Dict[int, np.ndarray] = {}

    # -- layouts -------------------------------------------------------------------------------
    def _xml(self, f, offset: int, size: int) -> ET.Element:
        f.seek(offset)
        return _strip_namespaces(ET.fromstring(f.read(size)))

    def _parse_v1(self, f) -> None:
        h = self.header
        self.xml = x = self._xml(f, int(h["XML_BLOCK_BYTE_OFFSET"]), int(h["XML_BLOCK_SIZE"]))
        self.signal_format = _text(x, "Data/SignalArrayFormat")
        if self.signal_format not in FORMATS:
            raise ValueError(f"unsupported CPHD signal array format {self.signal_format}")
        self.num_bytes_pvp = _int(x, "Data/NumBytesPVP")
        self.sign = int(_text(x, "Global/SGN", "-1"))
        pvp0, sig0 = int(h["PVP_BLOCK_BYTE_OFFSET"]), int(h["SIGNAL_BLOCK_BYTE_OFFSET"])
        self.channels = []
        for ch in x.findall("Data/Channel"):
            if ch.find("CompressionSize") is not None:
                raise NotImplementedError("compressed CPHD signal arrays are not supported")
            self.channels.append(CphdChannel(_text(ch, "Identifier", ""), _int(ch, "NumVectors"), _int(ch, "NumSamples"),
                                             sig0 + _int(ch, "SignalArrayByteOffset"),
                                             pvp0 + _int(ch, "PVPArrayByteOffset")))
        self.pvp_fields = {}
        pvp = x.find("PVP")
        for el in list(pvp) if pvp is not None else []:
            if el.tag == "AddedPVP":
                name = _text(el, "Name")
            else:
                name = el.tag
            off, size, fmt = _int(el, "Offset"), _int(el, "Size"), _text(el, "Format", "")
            count, dtype = _parse_pvp_format(fmt, size)
            self.pvp_fields[name] = PvpField(name, 8 * off, count, dtype)

    def _parse_v03(self, f) -> None:
        h = self.header
        self.xml = x = self._xml(f, int(h["XML_BYTE_OFFSET"]), int(h["XML_DATA_SIZE"]))
        st = _text(x, "Data/SampleType")
        if st not in SAMPLE_TYPES_03:
            raise ValueError(f"unsupported CPHD 0.3 sample type {st}")
        self.signal_format = SAMPLE_TYPES_03[st]
        self.num_bytes_pvp = _int(x, "Data/NumBytesVBP")
        self.sign = int(_text(x, "Global/PhaseSGN", "-1"))
        bps = FORMATS[self.signal_format][1]
        vb, sig = int(h["VB_BYTE_OFFSET"]), int(h["CPHD_BYTE_OFFSET"])
        self.channels = []
        for i, a in enumerate(x.findall("Data/ArraySize")):
            nv, ns = _int(a, "NumVectors"), _int(a, "NumSamples")
            self.channels.append(CphdChannel(str(i), nv, ns, sig, vb))
            vb += nv * self.num_bytes_pvp
            sig += nv * ns * bps
        self.pvp_fields = {}
        off = 0
        vp = x.find("VectorParameters")

        def walk(el):
            nonlocal off
            for c in el:
                if len(c):
                    walk(c)
                    continue
                size = int(c.text)
                ok = size % 8 == 0
                self.pvp_fields[c.tag] = PvpField(c.tag, off, size // 8 if ok else size, ">f8" if ok else None)
                off += size

        if vp is not None:
            walk(vp)

    # -- per-vector parameters -----------------------------------------------------------------
    def _pvp_array(self, index: int) -> np.ndarray:
        if index not in self._pvp_cache:
            ch = self.channels[index]
            names, formats, offsets = [], [], []
            for fld in self.pvp_fields.values():
                if fld.dtype is None:
                    continue
                names.append(fld.name)
                formats.append((fld.dtype, (fld.count,)) if fld.count > 1 else fld.dtype)
                offsets.append(fld.byte_offset)
            dt = np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": self.num_bytes_pvp})
            with open(self.path, "rb") as f:
                f.seek(ch.pvp_offset)
                buf = f.read(ch.num_vectors * self.num_bytes_pvp)
            if len(buf) != ch.num_vectors * self.num_bytes_pvp:
                raise ValueError("CPHD file is truncated (per-vector parameters)")
            self._pvp_cache[index] = np.frombuffer(buf, dtype=dt)
        return self._pvp_cache[index]

    def read_pvp_variable(self, variable: str, index: int = 0, the_range=None) -> Optional[np.ndarray]:
        """Values of one per-vector parameter of channel ``index`` (host float64 etc.): all vectors
        for None, vectors ``the_range`` for a slice, a one-element array for an int.  None when the
        file has no such parameter."""
        fld = self.pvp_fields.get(variable)
        if fld is None:
            return None
        if fld.dtype is None:
            raise NotImplementedError(f"PVP {variable} has a format this reader does not decode")
        arr = self._pvp_array(index)[variable]
        if the_range is None:
            sel = arr
        elif isinstance(the_range, (int, np.integer)):
            sel = arr[int(the_range):int(the_range) + 1]
        else:
            sel = arr[the_range]
        return np.ascontiguousarray(sel.astype(sel.dtype.newbyteorder("=")))

    # -- signal arrays -------------------------------------------------------------------------
    @property
    def bytes_per_sample(self) -> int:
        return FORMATS[self.signal_format][1]

    def _rows(self, item, n: int) -> np.ndarray:
        if item is None:
            item = slice(None)
        if isinstance(item, (int, np.integer)):
            i = int(item) + (n if item < 0 else 0)
            if not 0 <= i < n:
                raise IndexError("vector index out of range")
            return np.array([i])
        if isinstance(item, slice):
            return np.arange(n)[item]
        idx = np.asarray(item, dtype=np.int64).reshape(-1)
        if idx.size and (idx.min() < -n or idx.max() >= n):
            raise IndexError("vector index out of range")
        return np.where(idx < 0, idx + n, idx)

    def read_raw(self, item=slice(None), index: int = 0) -> np.ndarray:
        """Stored bytes of the selected vectors, [rows, NumSamples * bytes per sample] uint8."""
        ch = self.channels[index]
        rows = self._rows(item, ch.num_vectors)
        rb = ch.num_samples * self.bytes_per_sample
        out = np.empty((len(rows), rb), dtype=np.uint8)
        with open(self.path, "rb") as f:
            for j, r in enumerate(rows):
                f.seek(ch.signal_offset + int(r) * rb)
                if f.readinto(memoryview(out[j])) != rb:
                    raise ValueError("CPHD file is truncated (signal array)")
        return out

    def amp_sf(self, index: int = 0) -> Optional[np.ndarray]:
        return self.read_pvp_variable("AmpSF", index) if "AmpSF" in self.pvp_fields else None

    def read_device(self, item=slice(None), index: int = 0, device=None, apply_amp_sf: bool = True,
                    block_bytes: int = 64 << 20, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Selected vectors of channel ``index`` as a complex64 [rows, NumSamples] CUDA tensor,
        streamed from the file and decoded on the device (ordered on the current stream)."""
        dev = _device(device)
        ch = self.channels[index]
        rows = self._rows(item, ch.num_vectors)
        n, N = len(rows), ch.num_samples
        if out is None:
            out = torch.empty((n, N), dtype=torch.complex64, device=dev)
        elif out.shape != (n, N) or out.dtype != torch.complex64 or not out.is_contiguous() or out.device != dev:
            raise ValueError("out must be a contiguous complex64 tensor of the selected shape on the device")
        if n == 0 or N == 0:
            return out
        amp = self.amp_sf(index) if apply_amp_sf else None
        # contiguous runs of rows are streamed as they lie; other selections go row by row
        if np.all(np.diff(rows) == 1):
            runs = [(int(rows[0]), n, 0)]
        else:
            runs = [(int(r), 1, j) for j, r in enumerate(rows)]
        with torch.cuda.device(dev):
            amp_dev = None
            if amp is not None:
                amp_dev = torch.from_numpy(np.ascontiguousarray(amp[rows], dtype=np.float32)).to(dev, non_blocking=False)
            _stream_rows(self.path, ch.signal_offset, N * self.bytes_per_sample, FORMATS[self.signal_format][0], N,
                         runs, out, amp_dev, block_bytes)
        return out

    def read(self, item=slice(None), index: int = 0, apply_amp_sf: bool = True) -> np.ndarray:
        """Selected vectors as host complex64 [rows, NumSamples] (decoded on the current CUDA device)."""
        return self.read_device(item, index, apply_amp_sf=apply_amp_sf).cpu().numpy()


# -- streaming --------------------------------------------------------------------------------
_POOL: Optional[ThreadPoolExecutor] = None
_POOL_LOCK = threading.Lock()


def _read_threads() -> int:
    return max(1, min(16, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count() or 1))


def _pool() -> ThreadPoolExecutor:
    global _POOL
    with _POOL_LOCK:
        if _POOL is None:
            _POOL = ThreadPoolExecutor(max_workers=_read_threads(), thread_name_prefix="cphd-read")
        return _POOL


def _pread_full(fd: int, view: memoryview, offset: int) -> None:
    done = 0
    while done < len(view):
        got = os.preadv(fd, [view[done:]], offset + done)
        if got <= 0:
            raise ValueError("CPHD file is truncated (signal array)")
        done += got


def _pread_parallel(fd: int, view: memoryview, offset: int, pieces: int) -> None:
    n = len(view)
    if pieces <= 1 or n < (4 << 20):
        _pread_full(fd, view, offset)
        return
    step = -(-n // pieces)
    futs = [_pool().submit(_pread_full, fd, view[a:min(a + step, n)], offset + a) for a in range(0, n, step)]
    for fu in futs:
        fu.result()


def _device(device) -> torch.device:
    if device is None:
        return torch.device("cuda", torch.cuda.current_device())
    d = torch.device(device)
    return torch.device("cuda", torch.cuda.current_device()) if d.index is None else d


def _stream_rows(path: str, signal_offset: int, row_bytes: int, fmt_code: int, N: int, runs, out: torch.Tensor,
                 amp_dev: Optional[torch.Tensor], block_bytes: int) -> None:
    """Copy runs of rows (first file row, count, first output row) to ``out``: parallel reads into
    one of two pinned buffers while the other's copy and decode run on the device."""
    lib = _lib.load()
    dev = out.device
    compute = torch.cuda.current_stream(dev)
    copy = torch.cuda.Stream(dev)
    block_rows = max(1, block_bytes // row_bytes)
    cap = block_rows * row_bytes
    total_rows = sum(r[1] for r in runs)
    cap = min(cap, total_rows * row_bytes)
    pinned = [torch.empty(cap, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
    raw = [torch.empty(cap, dtype=torch.uint8, device=dev) for _ in range(2)]
    views = [memoryview(p.numpy()) for p in pinned]
    copied = [torch.cuda.Event() for _ in range(2)]
    decoded = [torch.cuda.Event() for _ in range(2)]
    pieces = _read_threads()
    blocks = []
    for r0, cnt, o0 in runs:
        for a in range(0, cnt, block_rows):
            blocks.append((r0 + a, min(block_rows, cnt - a), o0 + a))
    # the device buffers were allocated on the compute stream: earlier work there may still use
    # their memory, so the copy stream starts after it
    copy.wait_stream(compute)
    fd = os.open(path, os.O_RDONLY)
    try:
        for b, (fr, nr, orow) in enumerate(blocks):
            k = b & 1
            nb = nr * row_bytes
            if b >= 2:
                copied[k].synchronize()   # the host buffer's previous copy has left it
            _pread_parallel(fd, views[k][:nb], signal_offset + fr * row_bytes, pieces)
            with torch.cuda.stream(copy):
                if b >= 2:
                    copy.wait_event(decoded[k])   # the device buffer's previous decode has read it
                raw[k][:nb].copy_(pinned[k][:nb], non_blocking=True)
                copied[k].record(copy)
            compute.wait_event(copied[k])
            amp_ptr = None if amp_dev is None else amp_dev.data_ptr() + 4 * orow
            _lib.check(lib.sar_cphd_decode(ctypes.c_void_p(raw[k].data_ptr()), fmt_code, nr, N,
                                           ctypes.c_void_p(amp_ptr), ctypes.c_void_p(out[orow].data_ptr()),
                                           ctypes.c_void_p(compute.cuda_stream)), "sar_cphd_decode")
            decoded[k].record(compute)
    finally:
        os.close(fd)
    for t in raw:
        t.record_stream(copy)


# -- datasets -----------------------------------------------------------------------------------
class _CphdDataset:
    """One channel of a CPHD file as a dataset; the per-version parts are the class attributes."""

    _versions: Sequence[str] = ()
    _f0_name = ""
    _df_name = ""

    def __init__(self, file_address: str, channel_index: int = 0, c_eff: float = C,
                 waveform_fft: Optional[np.ndarray] = None, slow_time_weighting: Optional[np.ndarray] = None,
                 apply_amp_sf: bool = True, device=None):
        self._file_address = os.fspath(file_address)
        self._reader = CphdReader(self._file_address)
        if not any(self._reader.version.startswith(v) for v in self._versions):
            raise ValueError(f"{type(self).__name__} reads CPHD {'/'.join(self._versions)}, "
                             f"file is CPHD {self._reader.version}")
        if not 0 <= channel_index < len(self._reader.channels):
            raise IndexError("channel_index out of range")
        self._channel_index = channel_index
        self._waveform_fft = waveform_fft
        self._slow_time_weighting = slow_time_weighting
        self._c_eff = c_eff
        self._apply_amp_sf = apply_amp_sf
        self._device = device
        ch = self._reader.channels[channel_index]
        # as the reference: the channel's vectors, capped by the transmitter positions present
        self._num_slow_times = min(ch.num_vectors, self.transmitter_positions.shape[0])
        self._num_freqs = ch.num_samples
        self._sign_multiplier = 1.0 if self._reader.sign > 0 else -1.0

    @property
    def reader(self) -> CphdReader:
        if self._reader is None:
            self._reader = CphdReader(self._file_address)
        return self._reader

    @property
    def aperture(self) -> NumpySimpleSarAperture:
        return NumpySimpleSarAperture(self.transmitter_positions, self.receiver_positions, self.stab_ref_posns,
                                      self.centre_frequency, self.sample_bandwidth, self.waveform_fft,
                                      self.slow_time_weighting, num_freqs=None, sign_multiplier=self.sign_multiplier,
                                      c_eff=self.c_eff)

    @property
    def num_slow_times(self) -> int:
        return self._num_slow_times

    @property
    def num_freqs(self) -> int:
        return self._num_freqs

    def _pvp(self, name: str, the_range=slice(None)) -> np.ndarray:
        v = self.reader.read_pvp_variable(name, self._channel_index, the_range)
        if v is None:
            raise ValueError(f"CPHD file has no {name} per-vector parameter")
        return v

    @property
    def centre_frequency(self) -> float:
        """First sample frequency + half the sampled band (cphd101.py:101-114, cphd03.py:101-112)."""
        f0 = self._pvp(self._f0_name, 0)[0]
        delta_f = self._pvp(self._df_name, 0)[0]
        return float(f0 + 0.5 * (self.num_freqs * delta_f))

    @property
    def sample_bandwidth(self) -> float:
        return float(self.num_freqs * self._pvp(self._df_name, 0)[0])

    @property
    def transmitter_positions(self) -> np.ndarray:
        return self._pvp("TxPos")

    @property
    def receiver_positions(self) -> np.ndarray:
        return self._pvp("RcvPos")

    @property
    def stab_ref_posns(self) -> np.ndarray:
        return self._pvp("SRPPos")

    @property
    def waveform_fft(self) -> np.ndarray:
        if self._waveform_fft is None:
            self._waveform_fft = np.ones(self.num_freqs, dtype=np.complex128)
        return self._waveform_fft

    @property
    def slow_time_weighting(self) -> np.ndarray:
        if self._slow_time_weighting is None:
            self._slow_time_weighting = np.ones(self.num_slow_times, dtype=np.complex128)
        return self._slow_time_weighting

    @property
    def sign_multiplier(self) -> float:
        return self._sign_multiplier

    @property
    def c_eff(self) -> float:
        return self._c_eff

    def to_blocks(self, num_blocks: int = 1) -> List[NumpySimpleSarDataset]:
        """Apertures of ``num_blocks`` slow-time blocks without phase histories, as the reference's
        (cphd101.py:208-248): the last block takes the remainder."""
        def block(a, b):
            return NumpySimpleSarDataset.from_scratch(
                trans_posns=self.transmitter_positions[a:b, :], rec_posns=self.receiver_positions[a:b, :],
                srps=self.stab_ref_posns[a:b, :], centre_freq=self.centre_frequency,
                sample_freq=self.sample_bandwidth, waveform_fft=self.waveform_fft, num_freqs=self.num_freqs,
                sign_multiplier=self.sign_multiplier, slow_time_weighting=self.slow_time_weighting[a:b],
                c_eff=self.c_eff, phase_history=None)
        if num_blocks == 1:
            return [block(None, None)]
        n = self.num_slow_times // num_blocks
        return [block(i * n, self.num_slow_times if i == num_blocks - 1 else (i + 1) * n) for i in range(num_blocks)]

    def phase_history_device(self, item=slice(None), device=None, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Selected pulses as a complex64 CUDA tensor [rows, num_freqs], decoded on the device."""
        item = slice(0, self.num_slow_times) if item is None or item == slice(None) else item
        return self.reader.read_device(item, self._channel_index, device=device if device is not None else self._device,
                                       apply_amp_sf=self._apply_amp_sf, out=out)

    def phase_history(self, item=slice(None)) -> np.ndarray:
        """Selected pulses as host complex64 [rows, num_freqs] (cphd101.py:251-265)."""
        return self.phase_history_device(item).cpu().numpy()

    def get_subset(self, item: slice = None) -> NumpySimpleSarDataset:
        return NumpySimpleSarDataset(self.aperture.get_subset(item), self.phase_history(item))

    def __getstate__(self):
        state = dict(self.__dict__)
        state["_reader"] = None
        return state

    def __setstate__(self, state):
        self.__dict__ = state
        self._reader = CphdReader(self._file_address)


class Cphd101Dataset(_CphdDataset):
    """One channel of a CPHD 1.0.x file (io/cphd101.py:13-285): band from the SC0 / SCSS
    parameters, sign from Global/SGN."""
    _versions = ("1.",)
    _f0_name = "SC0"
    _df_name = "SCSS"


class Cphd03Dataset(_CphdDataset):
    """One channel of a CPHD 0.3 file (io/cphd03.py:13-289): band from the Fx0 / Fx_SS
    parameters, sign from Global/PhaseSGN."""
    _versions = ("0.3",)
    _f0_name = "Fx0"
    _df_name = "Fx_SS"


def open_phase_history(file_address: str, channel_index: int = 0, **kwargs) -> _CphdDataset:
    """The dataset class matching the file's CPHD version."""
    with open(file_address, "rb") as f:
        version, _ = read_header(f)
    cls = Cphd101Dataset if version.startswith("1.") else Cphd03Dataset if version.startswith("0.3") else None
    if cls is None:
        raise ValueError(f"unsupported CPHD version {version}")
    return cls(file_address, channel_index, **kwargs)


# -- writer -----------------------------------------------------------------------------------
_V1_PVP = [("TxTime", 1), ("TxPos", 3), ("TxVel", 3), ("RcvTime", 1), ("RcvPos", 3), ("RcvVel", 3), ("SRPPos", 3),
           ("aFDOP", 1), ("aFRR1", 1), ("aFRR2", 1), ("FX1", 1), ("FX2", 1), ("TOA1", 1), ("TOA2", 1),
           ("TDTropoSRP", 1), ("SC0", 1), ("SCSS", 1)]
_V03_VBP = [("TxTime", 1), ("TxPos", 3), ("RcvTime", 1), ("RcvPos", 3), ("SRPTime", 1), ("SRPPos", 3)]


def _quantise(ph: np.ndarray, fmt: str, amp_sf: bool):
    """(stored big-endian [S, 2N] array, per-vector AmpSF or None)."""
    comp = np.empty(ph.shape[:1] + (2 * ph.shape[1],), dtype=np.float64)
    comp[:, 0::2], comp[:, 1::2] = ph.real, ph.imag
    dt = FORMATS[fmt][2]
    if fmt == "CF8":
        return comp.astype(dt), (np.ones(ph.shape[0]) if amp_sf else None)
    top = float(np.iinfo(np.dtype(dt)).max)
    if amp_sf:
        a = np.abs(comp).max(axis=1) / top
        a[a == 0] = 1.0
        comp = comp / a[:, None]
    else:
        a = None
    return np.clip(np.rint(comp), -top, top).astype(dt), a


def _header(version: str, pairs: List[tuple]) -> bytes:
    return (f"CPHD/{version}\n" + "".join(f"{k} := {v}\n" for k, v in pairs)).encode("ascii") + SECTION_END


def _layout(version: str, keys: List[str], sizes: List[int], extra: List[tuple]) -> (bytes, List[int]):
    """Header with block offsets that account for its own length (fixed-width numbers)."""
    width = 20
    pairs = []
    for k in keys:
        pairs += [(f"{k}_SIZE" if version.startswith("1.") else k[0], "0" * width),
                  (f"{k}_BYTE_OFFSET" if version.startswith("1.") else k[1], "0" * width)]
    hlen = len(_header(version, pairs + extra))
    offs, pos = [], hlen
    for i, s in enumerate(sizes):
        pos = -(-pos // 8) * 8
        offs.append(pos)
        pos += s + (len(SECTION_END) if i == 0 else 0)   # the XML block is followed by a section end
    pairs = []
    for k, s, o in zip(keys, sizes, offs):
        pairs += [(f"{k}_SIZE" if version.startswith("1.") else k[0], str(s).zfill(width)),
                  (f"{k}_BYTE_OFFSET" if version.startswith("1.") else k[1], str(o).zfill(width))]
    return _header(version, pairs + extra), offs


def write_cphd(path: str, channels: Sequence[dict], version: str = "1.0.1", signal_format: str = "CF8",
               sign: int = -1, amp_sf: bool = False, added_pvp: Optional[Dict[str, np.ndarray]] = None) -> None:
    """Write a minimal CPHD file (the elements ``CphdReader`` reads; not schema-complete).

    ``channels``: dicts with ``phase_history`` [S, N] complex (natural frequency order, lowest
    first), ``trans_posns``, ``rec_posns``, ``srps`` [S, 3], ``centre_freq``, ``sample_bandwidth``
    and optionally ``identifier``, ``tx_times``.  Integer formats round the samples (after dividing
    by a per-vector AmpSF with ``amp_sf``, chosen so the largest component fills the type).
    ``added_pvp`` adds F8 per-vector parameters (CPHD 1.0 only), one array [S] per name, the
    same for every channel.
    """
    v1 = version.startswith("1.")
    if not v1 and not version.startswith("0.3"):
        raise ValueError("version must be 1.0.x or 0.3")
    if signal_format not in FORMATS:
        raise ValueError(f"signal_format must be one of {sorted(FORMATS)}")
    added_pvp = dict(added_pvp or {})
    if added_pvp and not v1:
        raise ValueError("added per-vector parameters need CPHD 1.0")
    fields = list(_V1_PVP if v1 else _V03_VBP)
    if amp_sf:
        fields.append(("AmpSF", 1))
    if not v1:
        fields += [("Fx0", 1), ("Fx_SS", 1), ("Fx1", 1), ("Fx2", 1)]
    fields += [(k, 1) for k in added_pvp]
    words = sum(c for _, c in fields)
    nbytes_pvp = 8 * words
    dt = np.dtype([(n, ">f8", (c,)) if c > 1 else (n, ">f8") for n, c in fields])
    pvp_parts, sig_parts, meta = [], [], []
    for ch in channels:
        ph = np.asarray(ch["phase_history"])
        S, N = ph.shape
        rec = np.zeros(S, dtype=dt)
        t = np.asarray(ch.get("tx_times", np.arange(S, dtype=np.float64)))
        fc, bw = float(ch["centre_freq"]), float(ch["sample_bandwidth"])
        df = bw / N
        f0 = fc - 0.5 * N * df
        stored, a = _quantise(ph, signal_format, amp_sf)
        for name, key in (("TxPos", "trans_posns"), ("RcvPos", "rec_posns"), ("SRPPos", "srps")):
            rec[name] = np.asarray(ch[key], dtype=np.float64)
        rec["TxTime"] = t
        rec["RcvTime"] = t
        if v1:
            rec["SC0"], rec["SCSS"], rec["FX1"], rec["FX2"] = f0, df, f0, f0 + (N - 1) * df
        else:
            rec["SRPTime"] = t
            rec["Fx0"], rec["Fx_SS"], rec["Fx1"], rec["Fx2"] = f0, df, f0, f0 + (N - 1) * df
        if amp_sf:
            rec["AmpSF"] = a
        for k, vals in added_pvp.items():
            rec[k] = np.asarray(vals, dtype=np.float64)
        pvp_parts.append(rec.tobytes())
        sig_parts.append(stored.tobytes())
        meta.append((ch.get("identifier", f"CH{len(meta)}"), S, N))
    pvp_block, sig_block = b"".join(pvp_parts), b"".join(sig_parts)
    if v1:
        pvp_xml, off = [], 0
        for n, c in fields:
            fmt = "X=F8;Y=F8;Z=F8;" if c == 3 else "F8"
            if n in added_pvp:
                pvp_xml.append(f"<AddedPVP><Name>{n}</Name><Offset>{off}</Offset><Size>{c}</Size><Format>{fmt}</Format></AddedPVP>")
            else:
                pvp_xml.append(f"<{n}><Offset>{off}</Offset><Size>{c}</Size><Format>{fmt}</Format></{n}>")
            off += c
        ch_xml, so, po = [], 0, 0
        for (ident, S, N) in meta:
            ch_xml.append(f"<Channel><Identifier>{ident}</Identifier><NumVectors>{S}</NumVectors>"
                          f"<NumSamples>{N}</NumSamples><SignalArrayByteOffset>{so}</SignalArrayByteOffset>"
                          f"<PVPArrayByteOffset>{po}</PVPArrayByteOffset></Channel>")
            so += S * N * FORMATS[signal_format][1]
            po += S * nbytes_pvp
        xml = (f'<?xml version="1.0" encoding="UTF-8"?><CPHD xmlns="http://api.nsgreg.nga.mil/schema/cphd/{version}">'
               f"<Global><DomainType>FX</DomainType><SGN>{int(sign)}</SGN></Global>"
               f"<Data><SignalArrayFormat>{signal_format}</SignalArrayFormat><NumBytesPVP>{nbytes_pvp}</NumBytesPVP>"
               f"<NumCPHDChannels>{len(meta)}</NumCPHDChannels>{''.join(ch_xml)}<NumSupportArrays>0</NumSupportArrays></Data>"
               f"<PVP>{''.join(pvp_xml)}</PVP></CPHD>").encode("utf-8")
        header, offs = _layout(version, ["XML_BLOCK", "PVP_BLOCK", "SIGNAL_BLOCK"],
                               [len(xml), len(pvp_block), len(sig_block)],
                               [("CLASSIFICATION", "UNCLASSIFIED"), ("RELEASE_INFO", "UNRESTRICTED")])
    else:
        st = {v: k for k, v in SAMPLE_TYPES_03.items()}[signal_format]
        vbp_xml = []
        for n, c in fields:
            if n == "Fx0":
                vbp_xml.append("<FxParameters>")
            vbp_xml.append(f"<{n}>{8 * c}</{n}>")
            if n == "Fx2":
                vbp_xml.append("</FxParameters>")
        arr = "".join(f"<ArraySize><NumVectors>{S}</NumVectors><NumSamples>{N}</NumSamples></ArraySize>" for _, S, N in meta)
        xml = ('<?xml version="1.0" encoding="UTF-8"?><CPHD xmlns="urn:CPHD:0.3">'
               f"<Global><DomainType>FX</DomainType><PhaseSGN>{int(sign)}</PhaseSGN></Global>"
               f"<Data><SampleType>{st}</SampleType><NumCPHDChannels>{len(meta)}</NumCPHDChannels>"
               f"<NumBytesVBP>{nbytes_pvp}</NumBytesVBP>{arr}</Data>"
               f"<VectorParameters>{''.join(vbp_xml)}</VectorParameters></CPHD>").encode("utf-8")
        header, offs = _layout(version, [("XML_DATA_SIZE", "XML_BYTE_OFFSET"), ("VB_DATA_SIZE", "VB_BYTE_OFFSET"),
                                         ("CPHD_DATA_SIZE", "CPHD_BYTE_OFFSET")],
                               [len(xml), len(pvp_block), len(sig_block)],
                               [("CLASSIFICATION", "UNCLASSIFIED"), ("RELEASE_INFO", "UNRESTRICTED")])
    with open(path, "wb") as f:
        f.write(header)
        for o, blob, tail in zip(offs, (xml, pvp_block, sig_block), (SECTION_END, b"", b"")):
            f.write(b"\0" * (o - f.tell()))
            f.write(blob + tail)
