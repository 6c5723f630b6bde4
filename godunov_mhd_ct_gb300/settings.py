"""Hot-path settings read from the reference's .ini decks.

Mirrors HydroSettings / MHDSettings (models/HydroSettings.cpp:18-31, models/MHDSettings.cpp:20):
same sections, keys and defaults, so an existing deck configures this path unchanged. The source
terms of the step read [gravity] enabled / uniform_gx, uniform_gy, uniform_gz (the keys of
app/test_mhd_rayleigh_taylor_3d.ini, read by kalypsso-core's get_uniform_gravity_vector) and
[viscosity] enabled / mu (app/test_mhd_kelvin_helmholtz_2d.ini, kalypsso-core's ViscosityParams);
the viscous Hancock predictor switch is [viscosity] hancock_predictor_enabled (off by default).
"""
from __future__ import annotations

import configparser
from dataclasses import dataclass

RIEMANN_IDS = {"UNKNOWN": 0, "APPROX": 1, "LLF": 2, "HLL": 3, "HLLC": 4, "HLLD": 5}


@dataclass
class MHDSettings:
    gamma0: float = 1.4
    cfl: float = 0.5
    slope_type: float = 1.0
    smallr: float = 1e-10
    smallc: float = 1e-10
    riemann: str = "UNKNOWN"
    small_beta: float = 1e-3
    scaling_factor: float = 1.0
    implementation_version: int = 0
    prolongation: str = "SIMPLE_COPY"  # [amr] cell_centered_prolongation_type
    time_integrator: str = "HANCOCK"  # [amr] time_integrator (HANCOCK or RK2_SSP)
    gravity: tuple | None = None  # [gravity] uniform (gx, gy, gz) when enabled
    viscosity_mu: float | None = None  # [viscosity] mu when enabled
    viscous_predictor: bool = False  # [viscosity] hancock_predictor_enabled

    @property
    def smallp(self) -> float:
        return self.smallc * self.smallc / self.gamma0

    @property
    def smallpp(self) -> float:
        return self.smallr * self.smallp

    @property
    def riemann_id(self) -> int:
        return RIEMANN_IDS.get(self.riemann.upper(), 0)

    @classmethod
    def from_ini(cls, text_or_path: str) -> "MHDSettings":
        """Parse an ini deck (a path or its text)."""
        cp = configparser.ConfigParser(inline_comment_prefixes=("#", ";"), strict=False)
        if "\n" in text_or_path or "[" in text_or_path:
            cp.read_string(text_or_path)
        else:
            with open(text_or_path) as f:
                cp.read_string(f.read())

        def get(sec, key, default, conv):
            if cp.has_option(sec, key):
                return conv(cp.get(sec, key).strip())
            return default

        def flag(v):
            return str(v).strip().lower() in ("1", "yes", "true", "on")

        gravity = None
        if flag(get("gravity", "enabled", "no", str)):
            gravity = tuple(get("gravity", "uniform_g" + c, 0.0, float) for c in "xyz")
        viscosity_mu = None
        if flag(get("viscosity", "enabled", "no", str)):
            viscosity_mu = get("viscosity", "mu", 0.0, float)

        return cls(
            gamma0=get("hydro", "gamma0", 1.4, float),
            cfl=get("hydro", "cfl", 0.5, float),
            slope_type=get("hydro", "slope_type", 1.0, float),
            smallr=get("hydro", "smallr", 1e-10, float),
            smallc=get("hydro", "smallc", 1e-10, float),
            riemann=get("hydro", "riemann", "UNKNOWN", str),
            small_beta=get("mhd", "small_beta", 1e-3, float),
            scaling_factor=get("mesh", "scaling_factor", 1.0, float),
            implementation_version=get("hydro", "implementation_version", 0, int),
            prolongation=get("amr", "cell_centered_prolongation_type", "SIMPLE_COPY", str),
            time_integrator=get("amr", "time_integrator", "HANCOCK", str),
            gravity=gravity,
            viscosity_mu=viscosity_mu,
            viscous_predictor=flag(get("viscosity", "hancock_predictor_enabled", "no", str)),
        )
