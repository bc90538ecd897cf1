"""FP64 populations of model atmospheres on the GPU.

The reference computes the per-layer populations, Doppler widths and the
molecular-equilibrium electron and mass densities of an ATLAS ``.atm`` model
in its converter before synthesis (``synthe_py/tools/convert_atm_to_npz.py``,
population stage ``:1860-2650``, with ``synthe_py/tools/pops_exact.py`` and
``synthe_py/tools/nmolec_exact.py``).  Here that stage runs on the GPU in FP64
(``ks_populations``): the ``.atm`` is parsed on the host as
``parse_atm_file`` does (``convert_atm_to_npz.py:190``), the abundances are
formed as the converter forms XABUND (``:1775-1800``), and the kernels return
the fields of the converted atmosphere that the synthesis reads
(``electron_density``, ``mass_density``, ``hckt``, ``xnf_h``, ``xnf_he1``,
``xnf_h2``, ``population_per_ion``, ``doppler_per_ion``).

There is no CPU fallback: every call needs the CUDA library.
"""

from __future__ import annotations

import ctypes as C
import math
import re
from dataclasses import replace
from pathlib import Path
from typing import Dict, List, Optional, Sequence, Union

import numpy as np
import torch

from .. import _native
from ..device import _require_cuda, stream_handle
from ..io.atmosphere import AtmosphereModel

N_ION = 6
N_SPECIES = 139
OUTPUT_FIELDS = ("electron_density", "mass_density", "hckt", "xnf_h", "xnf_he1", "xnf_h2",
                 "population_per_ion", "doppler_per_ion", "xnatm")


def parse_atm_file(atm_path: Union[str, Path]) -> dict:
    """Header values, abundances and the deck of an ATLAS ``.atm`` model
    (``convert_atm_to_npz.py:190-372``): ``teff``, ``glog``, ``title``,
    ``abundance_scale``, ``abundances`` {Z: value}, ``layers`` (one dict per
    row: RHOX, T, P, XNE, ABROSS, ACCRAD, VTURB)."""
    text = Path(atm_path).read_text(encoding="latin-1", errors="ignore").splitlines()
    data = {"teff": None, "glog": None, "title": None, "abundance_scale": 1.0, "abundances": {},
            "layers": []}
    i = 0
    while i < len(text):
        line = text[i].strip()
        if line.startswith("TEFF"):
            m = re.search(r"TEFF\s+([\d.]+)", line)
            if m:
                data["teff"] = float(m.group(1))
            m = re.search(r"(?:GRAVITY|LOG G)\s+([-\d.]+)", line)
            if not m:
                raise ValueError(f"{atm_path}: no GRAVITY on the TEFF line")
            data["glog"] = float(m.group(1))
        elif line.startswith("TITLE"):
            data["title"] = line[5:].strip()
        elif line.startswith("ABUNDANCE SCALE"):
            m = re.search(r"ABUNDANCE SCALE\s+([\d.]+)", line)
            if m:
                data["abundance_scale"] = float(m.group(1))
            parts = line.split("ABUNDANCE CHANGE")
            if len(parts) > 1:
                for z, a in re.findall(r"(\d+)\s+([+-]?\d+\.?\d*)", parts[1].strip()):
                    data["abundances"][int(z)] = float(a)
        elif line.startswith("ABUNDANCE CHANGE"):
            for z, a in re.findall(r"(\d+)\s+([+-]?\d+\.?\d*)", line):
                data["abundances"][int(z)] = float(a)
        elif line.startswith("READ DECK6"):
            i += 1
            break
        i += 1
    keys = ("RHOX", "T", "P", "XNE", "ABROSS", "ACCRAD", "VTURB")
    while i < len(text):
        parts = text[i].split()
        if len(parts) >= 7:
            data["layers"].append({k: float(v) for k, v in zip(keys, parts[:7])})
        i += 1
    if data["teff"] is None:
        raise ValueError(f"{atm_path}: could not parse TEFF")
    if data["glog"] is None:
        raise ValueError(f"{atm_path}: could not parse GRAVITY")
    if not data["layers"]:
        raise ValueError(f"{atm_path}: no layers after READ DECK6")
    return data


def abundance_vector(atm_data: dict) -> np.ndarray:
    """XABUND[99] as the converter forms it (``convert_atm_to_npz.py:1775-1800``):
    H and He as given (a negative value is a log10), the other elements
    ``abundance_scale * 10**log`` (missing elements: log = -20)."""
    out = np.zeros(99)
    scale = atm_data.get("abundance_scale", 1.0)
    for z in range(1, 100):
        a = atm_data["abundances"].get(z, -20.0)
        if z <= 2:
            out[z - 1] = 10.0 ** a if a < 0.0 else a
        else:
            la = math.log10(a) if a > 0.0 else a
            out[z - 1] = scale * (10.0 ** la)
    return out


def layer_columns(atm_data: dict) -> Dict[str, np.ndarray]:
    """RHOX, T, P and VTURB per layer (``convert_atm_to_npz.py:374-470``):
    RHOX given as log10 (negative first value) is exponentiated, and a gas
    pressure that is 1e5 x too small for hydrostatic equilibrium at the first
    layer is scaled by 1e6, as the converter does.  Layers must come in order
    of increasing RHOX."""
    rows = atm_data["layers"]
    rhox = np.array([r["RHOX"] for r in rows], dtype=np.float64)
    t = np.array([r["T"] for r in rows], dtype=np.float64)
    p = np.array([r["P"] for r in rows], dtype=np.float64)
    vt = np.array([r["VTURB"] for r in rows], dtype=np.float64)
    if rhox[0] < 0:
        rhox = 10.0 ** rhox
    if rhox.size > 1 and rhox[0] > rhox[-1]:
        raise ValueError("the model's layers must be in order of increasing RHOX")
    if p[0] > 0 and (10.0 ** atm_data["glog"]) * rhox[0] / p[0] > 1e5:
        p = p * 1e6
    return {"rhox": rhox, "temperature": t, "gas_pressure": p, "vturb": vt}


class DevicePopulations:
    """``ks_populations`` for one or more models: the inputs and every output in HBM.

    ``models`` are parsed ``.atm`` dicts (:func:`parse_atm_file`) or paths.
    ``run()`` enqueues the two kernels on ``stream`` and waits for them.
    """

    def __init__(self, models: Sequence[Union[dict, str, Path]], device="cuda"):
        L = _native.load()
        dev = _require_cuda(device)
        self.device = dev
        self.data: List[dict] = [m if isinstance(m, dict) else parse_atm_file(m) for m in models]
        self.inputs: List[Dict[str, torch.Tensor]] = []
        self.outputs: List[Dict[str, torch.Tensor]] = []
        self.iterations: List[torch.Tensor] = []
        self.rhox: List[np.ndarray] = []
        recs = (_native.KsPopsModel * len(self.data))()
        for k, d in enumerate(self.data):
            cols = layer_columns(d)
            n = cols["temperature"].size
            self.rhox.append(cols["rhox"])
            inp = {name: torch.from_numpy(np.ascontiguousarray(cols[name])).to(dev)
                   for name in ("temperature", "gas_pressure", "vturb")}
            inp["xabund"] = torch.from_numpy(abundance_vector(d)).to(dev)
            out = {name: torch.empty(n, dtype=torch.float64, device=dev)
                   for name in ("electron_density", "mass_density", "hckt", "xnf_h", "xnf_he1",
                                "xnf_h2", "xnatm")}
            out["population_per_ion"] = torch.empty((n, N_ION, N_SPECIES), dtype=torch.float64, device=dev)
            out["doppler_per_ion"] = torch.empty((n, N_ION, N_SPECIES), dtype=torch.float64, device=dev)
            it = torch.empty(n, dtype=torch.int32, device=dev)
            r = recs[k]
            r.n_layers = n
            r.temperature = inp["temperature"].data_ptr()
            r.gas_pressure = inp["gas_pressure"].data_ptr()
            r.vturb = inp["vturb"].data_ptr()
            r.xabund = inp["xabund"].data_ptr()
            for name in ("electron_density", "mass_density", "hckt", "xnf_h", "xnf_he1", "xnf_h2"):
                setattr(r, name, out[name].data_ptr())
            r.population = out["population_per_ion"].data_ptr()
            r.doppler = out["doppler_per_ion"].data_ptr()
            r.xnatom = out["xnatm"].data_ptr()
            r.nmolec_iterations = it.data_ptr()
            self.inputs.append(inp)
            self.outputs.append(out)
            self.iterations.append(it)
        self.recs = recs
        size = C.c_size_t(0)
        _native.check(L.ks_populations_workspace_size(recs, len(self.data), C.byref(size)))
        self.workspace = torch.empty(int(size.value) + 256, dtype=torch.uint8, device=dev)
        base = self.workspace.data_ptr()
        self._ws_ptr = (base + 255) & ~255
        self._ws_bytes = int(size.value)

    def run(self, stream: Optional[torch.cuda.Stream] = None) -> "DevicePopulations":
        L = _native.load()
        _native.check(L.ks_populations(self.recs, len(self.data), C.c_void_p(self._ws_ptr),
                                       self._ws_bytes, stream_handle(stream)))
        return self

    def host(self, k: int = 0) -> Dict[str, np.ndarray]:
        """The outputs of model ``k`` as host arrays (with ``depth``, ``temperature``,
        ``gas_pressure``, ``turbulent_velocity`` and the Newton iteration counts)."""
        out = {name: t.cpu().numpy() for name, t in self.outputs[k].items()}
        out["depth"] = self.rhox[k].copy()
        out["temperature"] = self.inputs[k]["temperature"].cpu().numpy()
        out["gas_pressure"] = self.inputs[k]["gas_pressure"].cpu().numpy()
        out["turbulent_velocity"] = self.inputs[k]["vturb"].cpu().numpy()
        out["nmolec_iterations"] = self.iterations[k].cpu().numpy()
        return out

    def atmosphere(self, k: int, continuum: AtmosphereModel) -> AtmosphereModel:
        """An :class:`AtmosphereModel` whose layers and populations are model ``k``'s
        GPU results and whose continuum coefficient tables come from ``continuum``
        (a converted model of the same atmosphere; the continuum opacity stage of
        the converter is not part of this library)."""
        h = self.host(k)
        if continuum.layers != h["temperature"].size:
            raise ValueError("the continuum model has a different number of layers")
        return replace(
            continuum,
            depth=h["depth"], temperature=h["temperature"], gas_pressure=h["gas_pressure"],
            turbulent_velocity=h["turbulent_velocity"], electron_density=h["electron_density"],
            mass_density=h["mass_density"], hckt=h["hckt"], xnf_h=h["xnf_h"], xnf_he1=h["xnf_he1"],
            xnf_h2=h["xnf_h2"], population_per_ion=h["population_per_ion"],
            doppler_per_ion=h["doppler_per_ion"],
        )


def compute_populations(atm_paths: Sequence[Union[str, Path, dict]], device="cuda") -> List[Dict[str, np.ndarray]]:
    """Populations of each model (host arrays), one batched GPU call."""
    pops = DevicePopulations(atm_paths, device=device).run()
    return [pops.host(k) for k in range(len(pops.data))]


def molecular_system() -> dict:
    """The molecular system built from the molecule table: number of molecules
    and equations, the element of each equation, and the elements whose
    populations come from the molecular equilibrium."""
    L = _native.load()
    nm, ne = C.c_int32(0), C.c_int32(0)
    eqe = np.zeros(32, dtype=np.int32)
    em = np.zeros(99, dtype=np.int32)
    _native.check(L.ks_pops_system(C.byref(nm), C.byref(ne), eqe.ctypes.data, em.ctypes.data))
    return {"n_molecules": int(nm.value), "n_equations": int(ne.value),
            "equation_element": eqe[:ne.value].copy(), "element_molecular": em.astype(bool)}


class PopulationTangents:
    """``ks_populations_tangent``: derivatives of model ``k`` of a
    :class:`DevicePopulations` with respect to the log10 abundances (dex) of
    ``elements`` (atomic numbers), one warp per element, all in one launch.
    ``run()`` fills ``d[field]`` ([n_elements, ...] device tensors) for the
    fields electron_density, mass_density, xnf_h, xnf_he1, xnf_h2 and
    population_per_ion at the model's current inputs."""

    FIELDS = ("electron_density", "mass_density", "xnf_h", "xnf_he1", "xnf_h2", "population_per_ion")

    def __init__(self, pops: DevicePopulations, k: int, elements: Sequence[int]):
        L = _native.load()
        self.pops, self.k = pops, k
        self.elements = [int(z) for z in elements]
        if any(z < 1 or z > 99 for z in self.elements):
            raise ValueError("elements are atomic numbers 1..99")
        n = pops.recs[k].n_layers
        dev = pops.device
        ne = len(self.elements)
        self.d = {f: torch.empty((ne, n), dtype=torch.float64, device=dev) for f in self.FIELDS[:-1]}
        self.d["population_per_ion"] = torch.empty((ne, n, N_ION, N_SPECIES), dtype=torch.float64, device=dev)
        recs = (_native.KsPopsTangent * ne)()
        base = pops.recs[k]
        for i, z in enumerate(self.elements):
            r = recs[i]
            r.model.n_layers = base.n_layers
            r.model.temperature = base.temperature
            r.model.gas_pressure = base.gas_pressure
            r.model.vturb = base.vturb
            r.model.xabund = base.xabund
            r.element = z - 1
            r.d_electron_density = self.d["electron_density"][i].data_ptr()
            r.d_mass_density = self.d["mass_density"][i].data_ptr()
            r.d_xnf_h = self.d["xnf_h"][i].data_ptr()
            r.d_xnf_he1 = self.d["xnf_he1"][i].data_ptr()
            r.d_xnf_h2 = self.d["xnf_h2"][i].data_ptr()
            r.d_population = self.d["population_per_ion"][i].data_ptr()
        self.recs = recs
        size = C.c_size_t(0)
        _native.check(L.ks_populations_tangent_workspace_size(recs, ne, C.byref(size)))
        self.workspace = torch.empty(int(size.value) + 256, dtype=torch.uint8, device=dev)
        self._ws_ptr = (self.workspace.data_ptr() + 255) & ~255
        self._ws_bytes = int(size.value)

    def run(self, stream: Optional[torch.cuda.Stream] = None) -> "PopulationTangents":
        L = _native.load()
        _native.check(L.ks_populations_tangent(self.recs, len(self.elements), C.c_void_p(self._ws_ptr),
                                               self._ws_bytes, stream_handle(stream)))
        return self
