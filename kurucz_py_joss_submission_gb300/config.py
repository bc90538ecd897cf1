"""Configuration records with the reference's field names
(synthe_py/config.py:12-134)."""

from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path
from typing import List, Optional, Tuple


@dataclass
class WavelengthGrid:
    start: float
    end: float
    resolution: float
    velocity_microturb: float = 0.0
    vacuum: bool = True


@dataclass
class LineDataConfig:
    atomic_catalog: Path
    molecular_catalogs: List[Path] = field(default_factory=list)
    include_predicted: bool = False
    cache_directory: Optional[Path] = None
    allow_tfort_runtime: bool = False


@dataclass
class AtmosphereInput:
    model_path: Path
    format: str = "atlas12"
    npz_path: Optional[Path] = None


@dataclass
class OutputConfig:
    spec_path: Path
    diagnostics_path: Optional[Path] = None


@dataclass
class SynthesisConfig:
    wavelength_grid: WavelengthGrid
    line_data: LineDataConfig
    atmosphere: AtmosphereInput
    output: OutputConfig
    cutoff: float = 1e-3
    linout: int = 30
    nlte: bool = False
    scattering_iterations: int = 8
    scattering_tolerance: float = 1e-3
    rhoxj_scale: float = 0.0
    log_level: str = "INFO"
    enable_helium_wings: bool = True
    skip_hydrogen_wings: bool = False
    line_filter: bool = True
    wavelength_subsample: int = 1
    n_workers: Optional[int] = None
    # GPU options of this implementation (no counterpart in the reference)
    precision: str = "mixed"
    tile_bins: int = 0
    warps_per_tile: int = 0
    # "npz": every atmosphere field from the converted model; "gpu": the
    # populations, Doppler widths, electron and mass densities recomputed from
    # the .atm model on the GPU (FP64), the continuum tables from the .npz
    populations: str = "npz"

    @classmethod
    def from_cli(
        cls,
        spec_path: Path,
        diagnostics_path: Optional[Path],
        atmosphere_path: Path,
        atomic_catalog: Path,
        wl_start: float,
        wl_end: float,
        resolution: float,
        velocity_microturb: float = 0.0,
        vacuum: bool = True,
        cutoff: float = 1e-3,
        linout: int = 30,
        nlte: bool = False,
        scattering_iterations: int = 8,
        scattering_tolerance: float = 1e-3,
        rhoxj_scale: float = 0.0,
        enable_helium_wings: bool = True,
        skip_hydrogen_wings: bool = False,
        line_filter: bool = True,
        wavelength_subsample: int = 1,
        npz_path: Optional[Path] = None,
        n_workers: Optional[int] = None,
        allow_tfort_runtime: bool = False,
        precision: str = "mixed",
        tile_bins: int = 0,
        warps_per_tile: int = 0,
        populations: str = "npz",
    ) -> "SynthesisConfig":
        return cls(
            wavelength_grid=WavelengthGrid(start=wl_start, end=wl_end, resolution=resolution,
                                           velocity_microturb=velocity_microturb, vacuum=vacuum),
            line_data=LineDataConfig(atomic_catalog=atomic_catalog,
                                     allow_tfort_runtime=allow_tfort_runtime),
            atmosphere=AtmosphereInput(model_path=atmosphere_path, npz_path=npz_path),
            output=OutputConfig(spec_path=spec_path, diagnostics_path=diagnostics_path),
            cutoff=cutoff, linout=linout, nlte=nlte,
            scattering_iterations=scattering_iterations,
            scattering_tolerance=scattering_tolerance, rhoxj_scale=rhoxj_scale,
            enable_helium_wings=enable_helium_wings, skip_hydrogen_wings=skip_hydrogen_wings,
            line_filter=line_filter, wavelength_subsample=wavelength_subsample,
            n_workers=n_workers, precision=precision, tile_bins=tile_bins,
            warps_per_tile=warps_per_tile, populations=populations,
        )


DEFAULT_WAVELENGTH: Tuple[float, float, float] = (300.0, 1800.0, 300_000.0)
