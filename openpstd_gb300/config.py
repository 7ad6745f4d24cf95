"""Scene configuration: a Python mirror of openPSTD's configuration classes.

Mirrors ``PSTDSettings``, ``DomainConfEdge``, ``DomainConf`` and
``PSTDConfiguration`` (kernel/KernelInterface.h:44-240,
kernel/KernelInterface.cpp:28-271 of the openPSTD tree) with the same method
names, so code written against the reference reads the same here.  Values are
kept as float32 where the reference stores ``float``; derived quantities
(``GetTimeStep``, ``GetWindowSize``) use the reference's arithmetic.

``to_c`` packs a configuration into the ``pstd_config`` struct of the C ABI
(include/pstd_gb300.h).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import List, Tuple

import numpy as np

f32 = np.float32

# kernel/core/kernel_functions.h:102-103
RK_COEFFICIENTS = [1.179799016570605e-1, 1.846469664911166e-1, 2.466236043095944e-1,
                   3.318395427360000e-1, 5e-1, 1.0]

# PSTD_DOMAIN_SIDE (kernel/KernelInterface.h:29-36)
PSTD_DOMAIN_SIDE_TOP = 1
PSTD_DOMAIN_SIDE_BOTTOM = 2
PSTD_DOMAIN_SIDE_LEFT = 4
PSTD_DOMAIN_SIDE_RIGHT = 8
PSTD_DOMAIN_SIDE_ALL = 15
PSTD_DOMAIN_SIDE_NONE = 0


PSTD_RECEIVERS_SPECTRAL = 2   # pstd_settings.spectral_interpolation value of spectral receivers


class PSTDSettings:
    """kernel/KernelInterface.h:44-158."""

    def __init__(self):
        self.calctime = f32(0)
        self.c1 = f32(0)
        self.ampMax = f32(0)
        self.freqMax = f32(0)
        self.rho = f32(0)
        self.patcherror = f32(0)
        self.tfactRK = f32(0)
        self.gridSpacing = f32(0)
        self.band_width = f32(0)
        self.wave_length = f32(0)
        self.rk_coefficients: List[float] = list(RK_COEFFICIENTS)
        self.spectral_interpolation = False
        # receivers: "nearest" (the reference: its spectral flag is read but the
        # interpolation is hard-disabled, kernel/core/Receiver.cpp:48) or
        # "spectral" (the point itself, windowed Fourier shifts along x then y)
        self.receiver_interpolation = "nearest"
        self.PMLCells = 0
        self.SaveNth = 1

    # getters / setters with the reference's names
    def GetGridSpacing(self): return self.gridSpacing
    def SetGridSpacing(self, v): self.gridSpacing = f32(v)
    def GetPatchError(self): return self.patcherror
    def SetPatchError(self, v): self.patcherror = f32(v)
    def GetRenderTime(self): return self.calctime
    def SetRenderTime(self, v): self.calctime = f32(v)
    def GetPMLCells(self): return self.PMLCells
    def SetPMLCells(self, v): self.PMLCells = int(v)
    def GetAttenuationOfPMLCells(self): return self.ampMax
    def SetAttenuationOfPMLCells(self, v): self.ampMax = f32(v)
    def GetDensityOfAir(self): return self.rho
    def SetDensityOfAir(self, v): self.rho = f32(v)
    def GetMaxFrequency(self): return self.freqMax
    def SetMaxFrequency(self, v): self.freqMax = f32(v)
    def GetSoundSpeed(self): return self.c1
    def SetSoundSpeed(self, v): self.c1 = f32(v)
    def GetFactRK(self): return self.tfactRK
    def SetFactRK(self, v): self.tfactRK = f32(v)
    def GetSaveNth(self): return self.SaveNth
    def SetSaveNth(self, v): self.SaveNth = int(v)
    def GetBandWidth(self): return self.band_width
    def SetBandWidth(self, v): self.band_width = f32(v)
    def GetSpectralInterpolation(self): return self.spectral_interpolation
    def SetSpectralInterpolation(self, v): self.spectral_interpolation = bool(v)
    def GetReceiverInterpolation(self): return self.receiver_interpolation

    def SetReceiverInterpolation(self, v):
        if v not in ("nearest", "spectral"):
            raise ValueError("receiver interpolation is 'nearest' or 'spectral'")
        self.receiver_interpolation = v

    def GetWaveLength(self): return self.wave_length
    def SetWaveLength(self, v): self.wave_length = f32(v)
    def GetRKCoefficients(self): return list(self.rk_coefficients)
    def SetRKCoefficients(self, c): self.rk_coefficients = [float(x) for x in c]

    def GetTimeStep(self):
        """dt = tfactRK * dx / c1 in float32 (kernel/KernelInterface.cpp:125-127)."""
        return f32(f32(self.tfactRK * self.gridSpacing) / self.c1)

    def GetWindowSize(self):
        """kernel/KernelInterface.cpp:128-134."""
        tmp = int(_round_half_away((float(self.patcherror) * 0.7 - 17) / 2.0))
        return int(_round_half_away(tmp * 2))

    def framecount(self) -> int:
        """Number of time steps, (int)(calctime/dt) (kernel/Solver.cpp:41)."""
        return int(f32(self.calctime) / self.GetTimeStep())


def _round_half_away(x: float) -> float:
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


@dataclass
class DomainConfEdge:
    """kernel/KernelInterface.h:163-175."""
    Absorption: float = 0.0
    LR: bool = False


@dataclass
class DomainConf:
    """kernel/KernelInterface.h:180-205; world coordinates in metres."""
    TopLeft: Tuple[float, float] = (0.0, 0.0)
    Size: Tuple[float, float] = (0.0, 0.0)
    T: DomainConfEdge = field(default_factory=DomainConfEdge)
    L: DomainConfEdge = field(default_factory=DomainConfEdge)
    B: DomainConfEdge = field(default_factory=DomainConfEdge)
    R: DomainConfEdge = field(default_factory=DomainConfEdge)

    def _edges(self, sides):
        out = []
        if sides & PSTD_DOMAIN_SIDE_TOP: out.append(self.T)
        if sides & PSTD_DOMAIN_SIDE_BOTTOM: out.append(self.B)
        if sides & PSTD_DOMAIN_SIDE_LEFT: out.append(self.L)
        if sides & PSTD_DOMAIN_SIDE_RIGHT: out.append(self.R)
        return out

    def GetAbsorption(self, side):
        e = self._edges(side)
        return e[0].Absorption if len(e) == 1 else 0.0

    def SetAbsorption(self, sides, absorption):
        for e in self._edges(sides):
            e.Absorption = float(absorption)

    def GetLR(self, side):
        e = self._edges(side)
        return e[0].LR if len(e) == 1 else False

    def SetLR(self, sides, lr):
        for e in self._edges(sides):
            e.LR = bool(lr)


class PSTDConfiguration:
    """kernel/KernelInterface.h:213-240."""

    def __init__(self):
        self.Settings = PSTDSettings()
        self.Speakers: List[Tuple[float, float, float]] = []
        self.Receivers: List[Tuple[float, float, float]] = []
        self.Domains: List[DomainConf] = []

    @staticmethod
    def CreateDefaultConf() -> "PSTDConfiguration":
        """kernel/KernelInterface.cpp:196-249."""
        conf = PSTDConfiguration()
        s = conf.Settings
        s.SetRenderTime(1.0)
        sound_speed, grid_spacing = 340.0, 0.2
        s.SetSoundSpeed(sound_speed)
        s.SetAttenuationOfPMLCells(20000.0)
        s.SetDensityOfAir(1.2)
        s.SetPatchError(70.0)
        s.SetFactRK(0.5)
        s.SetGridSpacing(grid_spacing)
        s.SetPMLCells(50)
        s.SetSaveNth(1)
        q = float(f32(sound_speed) / f32(grid_spacing))   # float / float in the reference
        s.SetBandWidth(3 * 1e-6 * q * q)
        s.SetRKCoefficients(RK_COEFFICIENTS)
        s.SetSpectralInterpolation(True)
        conf.Speakers.append((4.0, 5.0, 0.0))
        conf.Receivers.append((6.0, 5.0, 0.0))
        d = DomainConf((0.0, 0.0), (10.0, 15.0), DomainConfEdge(1, False), DomainConfEdge(0.3, False),
                       DomainConfEdge(0, False), DomainConfEdge(1, False))
        d2 = DomainConf((10.0, 4.0), (20.0, 15.0), DomainConfEdge(1, False), DomainConfEdge(1, False),
                        DomainConfEdge(0, False), DomainConfEdge(1, False))
        conf.Domains += [d, d2]
        return conf

    @staticmethod
    def CreateEmptyConf() -> "PSTDConfiguration":
        conf = PSTDConfiguration()
        conf.Settings.SetSaveNth(0)
        conf.Settings.SetSpectralInterpolation(False)
        return conf

    def copy(self) -> "PSTDConfiguration":
        import copy
        return copy.deepcopy(self)

    # ---- scene files: the PSTDConfiguration fields as JSON (Python floats
    # are written with enough digits to round-trip exactly)
    _SETTINGS = ["calctime", "c1", "ampMax", "freqMax", "rho", "patcherror", "tfactRK", "gridSpacing", "band_width",
                 "wave_length"]

    def to_dict(self) -> dict:
        s = self.Settings
        edge = lambda e: {"Absorption": float(e.Absorption), "LR": bool(e.LR)}
        return {
            "Settings": {**{k: float(getattr(s, k)) for k in self._SETTINGS},
                         "rk_coefficients": [float(x) for x in s.rk_coefficients],
                         "spectral_interpolation": bool(s.spectral_interpolation),
                         **({"receiver_interpolation": s.receiver_interpolation}
                            if s.receiver_interpolation != "nearest" else {}),
                         "PMLCells": int(s.PMLCells), "SaveNth": int(s.SaveNth)},
            "Domains": [{"TopLeft": [float(d.TopLeft[0]), float(d.TopLeft[1])],
                         "Size": [float(d.Size[0]), float(d.Size[1])],
                         "T": edge(d.T), "L": edge(d.L), "B": edge(d.B), "R": edge(d.R)} for d in self.Domains],
            "Speakers": [[float(v) for v in p] for p in self.Speakers],
            "Receivers": [[float(v) for v in p] for p in self.Receivers],
        }

    @staticmethod
    def from_dict(d: dict) -> "PSTDConfiguration":
        conf = PSTDConfiguration()
        s, src = conf.Settings, d["Settings"]
        for k in PSTDConfiguration._SETTINGS:
            setattr(s, k, f32(src[k]))
        s.rk_coefficients = [float(x) for x in src["rk_coefficients"]]
        s.spectral_interpolation = bool(src.get("spectral_interpolation", False))
        s.SetReceiverInterpolation(src.get("receiver_interpolation", "nearest"))
        s.PMLCells = int(src["PMLCells"])
        s.SaveNth = int(src["SaveNth"])
        edge = lambda e: DomainConfEdge(float(e["Absorption"]), bool(e["LR"]))
        conf.Domains = [DomainConf((float(x["TopLeft"][0]), float(x["TopLeft"][1])),
                                   (float(x["Size"][0]), float(x["Size"][1])),
                                   edge(x["T"]), edge(x["L"]), edge(x["B"]), edge(x["R"])) for x in d["Domains"]]
        conf.Speakers = [tuple(float(v) for v in p) for p in d["Speakers"]]
        conf.Receivers = [tuple(float(v) for v in p) for p in d["Receivers"]]
        return conf

    def save(self, path: str):
        import json
        with open(path, "w") as f:
            json.dump(self.to_dict(), f, indent=1)

    @staticmethod
    def load(path: str) -> "PSTDConfiguration":
        import json
        with open(path) as f:
            return PSTDConfiguration.from_dict(json.load(f))


# ---------------------------------------------------------------------------
# ctypes mirror of include/pstd_gb300.h
class c_settings(ctypes.Structure):
    _fields_ = [("calctime", ctypes.c_float), ("c1", ctypes.c_float), ("ampMax", ctypes.c_float),
                ("freqMax", ctypes.c_float), ("rho", ctypes.c_float), ("patcherror", ctypes.c_float),
                ("tfactRK", ctypes.c_float), ("gridSpacing", ctypes.c_float), ("band_width", ctypes.c_float),
                ("wave_length", ctypes.c_float), ("rk_coefficients", ctypes.c_float * 6),
                ("n_rk_coefficients", ctypes.c_int32), ("spectral_interpolation", ctypes.c_int32),
                ("PMLCells", ctypes.c_int32), ("SaveNth", ctypes.c_int32)]


class c_edge(ctypes.Structure):
    _fields_ = [("absorption", ctypes.c_float), ("lr", ctypes.c_int32)]


class c_domain_conf(ctypes.Structure):
    _fields_ = [("top_left", ctypes.c_float * 2), ("size", ctypes.c_float * 2),
                ("T", c_edge), ("L", c_edge), ("B", c_edge), ("R", c_edge)]


class c_config(ctypes.Structure):
    _fields_ = [("settings", c_settings), ("n_domains", ctypes.c_int32),
                ("domains", ctypes.POINTER(c_domain_conf)), ("n_speakers", ctypes.c_int32),
                ("speakers", ctypes.POINTER(ctypes.c_float)), ("n_receivers", ctypes.c_int32),
                ("receivers", ctypes.POINTER(ctypes.c_float))]


class c_domain_info(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int32), ("top_left", ctypes.c_int32 * 2), ("size", ctypes.c_int32 * 2),
                ("is_pml", ctypes.c_int32), ("is_secondary_pml", ctypes.c_int32), ("is_rigid", ctypes.c_int32),
                ("local", ctypes.c_int32), ("should_update", ctypes.c_int32 * 2),
                ("n_neighbours", ctypes.c_int32 * 4), ("fft_length", ctypes.c_int32 * 2),
                ("window", ctypes.c_int32 * 2), ("alpha", ctypes.c_float), ("impedance", ctypes.c_float),
                ("rho", ctypes.c_float)]

    def as_dict(self):
        return {
            "id": self.id, "top_left": tuple(self.top_left), "size": tuple(self.size),
            "is_pml": bool(self.is_pml), "is_secondary_pml": bool(self.is_secondary_pml),
            "is_rigid": bool(self.is_rigid), "local": bool(self.local),
            "should_update": tuple(bool(x) for x in self.should_update),
            "n_neighbours": tuple(self.n_neighbours), "fft_length": tuple(self.fft_length),
            "window": tuple(self.window), "alpha": self.alpha, "impedance": self.impedance, "rho": self.rho,
        }


class CConfig:
    """Owns a ``pstd_config`` and the arrays it points to."""

    def __init__(self, conf: PSTDConfiguration):
        s = conf.Settings
        st = c_settings()
        st.calctime = float(s.calctime); st.c1 = float(s.c1); st.ampMax = float(s.ampMax)
        st.freqMax = float(s.freqMax); st.rho = float(s.rho); st.patcherror = float(s.patcherror)
        st.tfactRK = float(s.tfactRK); st.gridSpacing = float(s.gridSpacing)
        st.band_width = float(s.band_width); st.wave_length = float(s.wave_length)
        rk = list(s.rk_coefficients)
        for i in range(min(6, len(rk))):
            st.rk_coefficients[i] = float(rk[i])
        st.n_rk_coefficients = len(rk)
        st.spectral_interpolation = (PSTD_RECEIVERS_SPECTRAL if s.receiver_interpolation == "spectral"
                                     else int(bool(s.spectral_interpolation)))
        st.PMLCells = int(s.PMLCells); st.SaveNth = int(s.SaveNth)
        n = len(conf.Domains)
        self._domains = (c_domain_conf * max(1, n))()
        for i, d in enumerate(conf.Domains):
            cd = self._domains[i]
            cd.top_left[0], cd.top_left[1] = float(d.TopLeft[0]), float(d.TopLeft[1])
            cd.size[0], cd.size[1] = float(d.Size[0]), float(d.Size[1])
            for name in ("T", "L", "B", "R"):
                e = getattr(d, name)
                setattr(cd, name, c_edge(float(e.Absorption), int(bool(e.LR))))
        spk = [float(v) for p in conf.Speakers for v in (list(p) + [0.0] * (3 - len(p)))]
        rec = [float(v) for p in conf.Receivers for v in (list(p) + [0.0] * (3 - len(p)))]
        self._spk = (ctypes.c_float * max(1, len(spk)))(*spk)
        self._rec = (ctypes.c_float * max(1, len(rec)))(*rec)
        self.c = c_config(st, n, self._domains, len(conf.Speakers), self._spk, len(conf.Receivers), self._rec)

    def ptr(self):
        return ctypes.byref(self.c)
