"""Variogram model description shared by every entry point.

Mirrors ``VariogramModel`` / ``Structure`` / ``Anisotropy`` of the reference
(crates/geostat-core/src/variogram/model.rs:288-630), including its serde
JSON layout (``{"nugget": .., "structures": [{"kind": "spherical", "sill": ..,
"range": .., "anis": {..}}]}``) and the validation of
``VariogramModel::new`` (model.rs:554-630), so a model file written by the
geostat CLI loads unchanged.
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass, field
from typing import List, Optional

from .errors import InvalidParameter

# Kind codes shared with the C ABI (include/geostat_gb300.h, GS_KIND_*).
KIND_CODES = {
    "spherical": 0, "exponential": 1, "gaussian": 2, "matern15": 3, "matern25": 4,
    "circular": 5, "stable": 6, "hole": 7, "wave": 8, "power": 9,
}
# Kinds the CUDA path evaluates (closed forms); model.rs:122-141.
GPU_KINDS = ("spherical", "exponential", "gaussian", "matern15", "matern25")

_ALIASES = {
    "sph": "spherical", "spherical": "spherical", "exp": "exponential",
    "exponential": "exponential", "gau": "gaussian", "gaussian": "gaussian",
    "mat15": "matern15", "matern15": "matern15", "mat25": "matern25", "matern25": "matern25",
    "cir": "circular", "circular": "circular", "hol": "hole", "hole": "hole",
    "wav": "wave", "wave": "wave",
}


def parse_kind(spec: str):
    """``ModelKind::from_str`` (model.rs:215-279): returns ``(kind, param)``."""
    s = spec.strip().lower()
    if s in _ALIASES:
        return _ALIASES[s], 0.0
    for prefix, kind in (("stable:", "stable"), ("power:", "power")):
        if s.startswith(prefix):
            try:
                p = float(s[len(prefix):])
            except ValueError:
                raise InvalidParameter(f"invalid {kind} parameter '{s[len(prefix):]}'")
            return kind, p
    raise InvalidParameter(f"unknown model kind '{spec}'")


@dataclass
class Anisotropy:
    """GSLIB/gstat geometric anisotropy (model.rs:288-340)."""
    azimuth_deg: float
    ratio: float
    ratio_z: float = 1.0
    dip_deg: float = 0.0
    rake_deg: float = 0.0

    def validate(self):
        """``Anisotropy::validate`` (model.rs:378-405)."""
        if not (self.ratio_z > 0.0) or not math.isfinite(self.ratio_z):
            raise InvalidParameter(f"anisotropy ratio_z must be finite and > 0, got {self.ratio_z}")
        if not (self.ratio > 0.0) or not math.isfinite(self.ratio):
            raise InvalidParameter(f"anisotropy ratio must be finite and > 0, got {self.ratio}")
        if not math.isfinite(self.azimuth_deg):
            raise InvalidParameter("anisotropy azimuth must be finite")
        if not math.isfinite(self.dip_deg) or not math.isfinite(self.rake_deg):
            raise InvalidParameter("anisotropy dip/rake must be finite")

    def to_dict(self):
        d = {"azimuth_deg": self.azimuth_deg, "ratio": self.ratio}
        if self.ratio_z != 1.0:
            d["ratio_z"] = self.ratio_z
        if self.dip_deg != 0.0:
            d["dip_deg"] = self.dip_deg
        if self.rake_deg != 0.0:
            d["rake_deg"] = self.rake_deg
        return d


@dataclass
class Structure:
    """One nested structure (model.rs:436-519)."""
    kind: str
    sill: float
    range: float
    anis: Optional[Anisotropy] = None
    param: float = 0.0

    def __post_init__(self):
        if self.kind not in KIND_CODES:
            self.kind, p = parse_kind(self.kind)
            if p:
                self.param = p

    @staticmethod
    def with_anisotropy(kind, sill, range_, azimuth_deg, ratio):
        return Structure(kind, sill, range_, Anisotropy(azimuth_deg, ratio))

    @staticmethod
    def with_rotation(kind, sill, range_, azimuth_deg, dip_deg, rake_deg, ratio, ratio_z):
        return Structure(kind, sill, range_, Anisotropy(azimuth_deg, ratio, ratio_z, dip_deg,
                                                        rake_deg))

    def kind_json(self):
        if self.kind in ("stable", "power"):
            return {self.kind: self.param}
        return self.kind


@dataclass
class VariogramModel:
    """Nugget plus nested structures; validated like ``VariogramModel::new``."""
    nugget: float
    structures: List[Structure] = field(default_factory=list)

    def __post_init__(self):
        self.validate()

    def validate(self):
        if not (self.nugget >= 0.0) or not math.isfinite(self.nugget):
            raise InvalidParameter(f"nugget must be finite and >= 0, got {self.nugget}")
        if len(self.structures) > 4:
            raise InvalidParameter("at most 4 nested structures are supported")
        for s in self.structures:
            if not (s.sill >= 0.0) or not math.isfinite(s.sill):
                raise InvalidParameter(f"partial sill must be finite and >= 0, got {s.sill}")
            if not (s.range > 0.0) or not math.isfinite(s.range):
                raise InvalidParameter(f"range must be finite and > 0, got {s.range}")
            if s.kind == "stable" and (not (s.param > 0.0) or s.param > 2.0):
                raise InvalidParameter(f"Stable alpha must be in (0, 2], got {s.param}")
            if s.kind == "power" and (not (s.param > 0.0) or s.param >= 2.0):
                raise InvalidParameter(f"Power theta must be in (0, 2), got {s.param}")
            if s.anis is not None:
                s.anis.validate()
        if not (self.total_sill() > 0.0):
            raise InvalidParameter("total sill must be positive")

    def total_sill(self) -> float:
        return self.nugget + sum(s.sill for s in self.structures)

    def has_power(self) -> bool:
        return any(s.kind == "power" for s in self.structures)

    def gpu_supported(self) -> bool:
        return all(s.kind in GPU_KINDS for s in self.structures)

    # -- serde JSON layout of the reference ---------------------------------
    def to_json(self) -> str:
        out = {"nugget": self.nugget, "structures": []}
        for s in self.structures:
            d = {"kind": s.kind_json(), "sill": s.sill, "range": s.range}
            if s.anis is not None:
                d["anis"] = s.anis.to_dict()
            out["structures"].append(d)
        return json.dumps(out)

    @staticmethod
    def from_json(text: str) -> "VariogramModel":
        raw = json.loads(text)
        structs = []
        for d in raw.get("structures", []):
            k = d["kind"]
            param = 0.0
            if isinstance(k, dict):
                (k, param), = k.items()
                k = k.lower()
            a = d.get("anis")
            anis = None
            if a is not None:
                anis = Anisotropy(a["azimuth_deg"], a["ratio"], a.get("ratio_z", 1.0),
                                  a.get("dip_deg", 0.0), a.get("rake_deg", 0.0))
            structs.append(Structure(k, float(d["sill"]), float(d["range"]), anis, float(param)))
        return VariogramModel(float(raw["nugget"]), structs)

    def __repr__(self):
        parts = [f"{self.nugget:.4f} Nug"]
        for s in self.structures:
            parts.append(f"{s.sill:.4f} {s.kind}({s.range:.1f})")
        return "VariogramModel(" + " + ".join(parts) + ")"
