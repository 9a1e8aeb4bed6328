"""Visual-flocking parameters (VFParams) and the reference's .env keys.

Mirrors the reference's parameter bundle ``abm/projects/visual_flocking/vf_contrib/vf_params.py:9-23``
(GAM, V0, ALP0/1/2, BET0/1/2, BOUNDARY, LIMIT_MOVEMENT, MAX_VEL, MAX_TH) plus the simulation
geometry of ``abm/simulation/sims.py:60-161`` (arena, window pad, FOV, VPF resolution, agent
radius).  ``from_env`` reads the same keys as the reference, including its quirk that GAM is
read from ``VF_GAMMA`` while the shipped .env files set ``VF_GAM`` (so GAM stays 0.1).
"""
from __future__ import annotations

import dataclasses
import math

from . import _lib


@dataclasses.dataclass
class VFParams:
    gam: float = 0.1
    v0: float = 1.0
    alp0: float = 1.0
    alp1: float = 0.09
    alp2: float = 0.0
    bet0: float = 1.0
    bet1: float = 0.09
    bet2: float = 0.0
    boundary: str = "walls"          # "walls" | "infinite"
    limit_movement: bool = False
    max_vel: float = 3.0
    max_th: float = 0.1
    width: float = 600.0
    height: float = 480.0
    window_pad: float = 30.0
    fov: tuple = (-math.pi, math.pi)
    rv: int = 800
    radius: float = 10.0
    dt: float = 1.0

    # reference attribute names (vf_params.GAM ...), for duck-typed callers
    GAM = property(lambda s: s.gam)
    V0 = property(lambda s: s.v0)
    ALP0 = property(lambda s: s.alp0)
    ALP1 = property(lambda s: s.alp1)
    ALP2 = property(lambda s: s.alp2)
    BET0 = property(lambda s: s.bet0)
    BET1 = property(lambda s: s.bet1)
    BET2 = property(lambda s: s.bet2)

    def to_c(self) -> _lib.AbmVfParams:
        if self.boundary not in ("walls", "infinite"):
            raise ValueError(f"boundary must be 'walls' or 'infinite', got {self.boundary!r}")
        return _lib.AbmVfParams(
            gam=self.gam, v0=self.v0, alp0=self.alp0, alp1=self.alp1, alp2=self.alp2,
            bet0=self.bet0, bet1=self.bet1, bet2=self.bet2,
            boundary=1 if self.boundary == "infinite" else 0,
            limit_movement=1 if self.limit_movement else 0, max_vel=self.max_vel,
            max_th=self.max_th, width=self.width, height=self.height,
            window_pad=self.window_pad, fov0=float(self.fov[0]), fov1=float(self.fov[1]),
            rv=int(self.rv), reserved0=0, radius=self.radius, dt=self.dt)

    def oracle_dict(self) -> dict:
        """Flat dict in the oracle's parameter slots (tests only)."""
        return dict(gam=self.gam, v0=self.v0, alp0=self.alp0, alp1=self.alp1, alp2=self.alp2,
                    bet0=self.bet0, bet1=self.bet1, bet2=self.bet2,
                    boundary=1 if self.boundary == "infinite" else 0,
                    limit_movement=1 if self.limit_movement else 0, max_vel=self.max_vel,
                    max_th=self.max_th, width=self.width, height=self.height,
                    window_pad=self.window_pad, fov0=self.fov[0], fov1=self.fov[1],
                    rv=self.rv, radius=self.radius, dt=self.dt)

    @classmethod
    def from_env(cls, env: dict, **over) -> "VFParams":
        """Build from a reference .env mapping (dotenv_values output)."""
        g = lambda k, d: env.get(k, d)
        fov_ratio = float(g("AGENT_FOV", 1.0))
        rv = int(float(g("VISUAL_FIELD_RESOLUTION", 800)))
        rv = int(rv * (1 / fov_ratio))      # VFSimulation rescale, vf_sims.py:40-44
        p = cls(gam=float(g("VF_GAMMA", 0.1)), v0=float(g("VF_V0", 1)),
                alp0=float(g("VF_ALP0", 1)), alp1=float(g("VF_ALP1", 0.09)),
                alp2=float(g("VF_ALP2", 0)), bet0=float(g("VF_BET0", 1)),
                bet1=float(g("VF_BET1", 0.09)), bet2=float(g("VF_BET2", 0)),
                boundary=g("BOUNDARY", "walls"),
                limit_movement=bool(float(g("VF_LIMIT_MOVEMENT", "0"))),
                max_vel=float(g("VF_MAX_VEL", "3")), max_th=float(g("VF_MAX_TH", "0.1")),
                width=float(g("ENV_WIDTH", 600)), height=float(g("ENV_HEIGHT", 480)),
                fov=(-fov_ratio * math.pi, fov_ratio * math.pi), rv=rv,
                radius=float(g("RADIUS_AGENT", 10)))
        return dataclasses.replace(p, **over)
