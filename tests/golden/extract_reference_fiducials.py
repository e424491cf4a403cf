"""Extract the golden vectors of the reference's unit tests into reference_fiducials.json.

Run where the reference source tree is present (the argument, else $CHOLLA_REFERENCE, else a
directory named `reference` beside the repository):

    python tests/golden/extract_reference_fiducials.py [/path/to/cholla]

Only numbers are taken from the reference's test files (fiducial outputs and the literal
inputs of the small known-answer tests); the inputs of the randomised tests are regenerated
by the oracle's std::mt19937_64 / std::mt19937 helpers with the seeds and ranges recorded here.
"""
from __future__ import annotations

import json
import math
import os
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def braces_to_json(text: str):
    t = re.sub(r"//[^\n]*", "", text)
    t = t.replace("{", "[").replace("}", "]")
    t = re.sub(r",\s*]", "]", t)
    return json.loads(t)


def initializer(src: str, name: str, start: int = 0) -> tuple[object, int]:
    """JSON value of `<type> name = {...};` (or `name{...};`) found at or after `start`."""
    m = re.compile(re.escape(name) + r"\s*(=\s*)?\{").search(src, start)
    if not m:
        raise KeyError(name)
    i = src.index("{", m.start())
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                return braces_to_json(src[i:j + 1]), j
    raise ValueError(name)


def split_mhd(block: str) -> tuple[str, str]:
    """(MHD branch, hydro branch) of an `#ifdef MHD ... #else ... #endif` region."""
    m = re.search(r"#ifdef MHD(.*?)#else[^\n]*\n(.*?)#endif", block, re.S)
    return m.group(1), m.group(2)


def maps(lst) -> list[dict]:
    return [{str(int(k)): float(v) for k, v in d} for d in lst]


def ppmc_vl(src_dir: Path) -> dict:
    s = (src_dir / "reconstruction/ppmc_cuda_tests.cu").read_text()
    t0 = s.index("TEST(tALLPpmcVLReconstructor")
    body = s[t0:s.index("// Loop over different directions", t0)]
    mhd, hydro = split_mhd(body[body.index("// Fiducial Data"):])
    out = {}
    for tag, b in (("mhd", mhd), ("hydro", hydro)):
        left, _ = initializer(b, "fiducial_interface_left")
        right, _ = initializer(b, "fiducial_interface_right")
        out[tag] = {"left": maps(left), "right": maps(right)}
    out["setup"] = {"seed": 42, "range": [0.1, 5.0], "nx": 6, "ny": 6, "nz": 6, "gamma": 5.0 / 3.0,
                    "n_fields": {"hydro": 5, "mhd": 8}, "source": "src/reconstruction/ppmc_cuda_tests.cu:121-259"}
    return out


def plmc(src_dir: Path) -> dict:
    s = (src_dir / "reconstruction/plmc_cuda_tests.cu").read_text()
    out = {}
    for test, tag in (("TEST(tHYDROPlmcReconstructor", "hydro"), ("TEST(tMHDPlmcReconstructor", "mhd")):
        if test not in s:
            continue
        t0 = s.index(test)
        left, j = initializer(s, "fiducial_interface_left", t0)
        right, _ = initializer(s, "fiducial_interface_right", j)
        head = s[t0:s.index("fiducial_interface_left", t0)]
        dims = {}
        for k in ("nx", "ny", "nz", "n_fields"):
            m = re.search(rf"\b{k}\s*=\s*(\w+)", head)
            v = m.group(1)
            dims[k] = int(v) if v.isdigit() else dims[v]
        out[tag] = {"left": maps(left), "right": maps(right), **dims}
    out["setup"] = {"seed": 42, "range": [0.1, 5.0], "gamma": 5.0 / 3.0, "draws_before_grid": 2,
                    "source": "src/reconstruction/plmc_cuda_tests.cu:26-293"}
    return out


def ppm_single_variable(src_dir: Path) -> dict:
    s = (src_dir / "reconstruction/reconstruction_tests.cu").read_text()
    t0 = s.index("TEST(tALLReconstructionPPMSingleVariable")
    left, j = initializer(s, "fiducial_left_interface", t0)
    right, _ = initializer(s, "fiducial_right_interface", j)
    return {"seed": 42, "range": [-100.0, 100.0], "n_tests": 100, "left": left, "right": right,
            "source": "src/reconstruction/reconstruction_tests.cu:501-572"}


def dt_tests(src_dir: Path) -> dict:
    s = (src_dir / "hydro/hydro_cuda_tests.cu").read_text()
    t0 = s.index("TEST(tHYDROCalcDt3D")
    blk = s[t0:s.index("TEST(", t0 + 10)]
    vals = [float(v) for v in re.findall(r"host_conserved\.at\(\d\)\s*=\s*([-0-9.eE]+)", blk)]
    calc = {"conserved": vals, "gamma": 5.0 / 3.0, "dx": 1.0, "dy": 1.0, "dz": 1.0,
            "fiducial": float(re.search(r"fiducialDt\s*=\s*([-0-9.eE]+)", blk).group(1)),
            "source": "src/hydro/hydro_cuda_tests.cu:29-82"}
    t1 = s.index("TEST(tHYDROHydroInverseCrossingTime")
    blk = s[t1:s.index("TEST(", t1 + 10)]
    names = ["energy", "density", "velocityX", "velocityY", "velocityZ", "cellSizeX", "cellSizeY", "cellSizeZ"]
    ict = {n: float(re.search(rf"double const {n}\s*=\s*([-0-9.eE]+)", blk).group(1)) for n in names}
    ict["fiducial"] = float(re.search(r"fiducialInverseCrossingTime\s*=\s*([-0-9.eE]+)", blk).group(1))
    ict["gamma"] = 5.0 / 3.0
    ict["source"] = "src/hydro/hydro_cuda_tests.cu:89-110"
    t2 = s.index("TEST(tMHDMhdInverseCrossingTime")
    blk = s[t2:s.index("TEST(", t2 + 10)]
    names += ["magneticX", "magneticY", "magneticZ"]
    mct = {n: float(re.search(rf"double const {n}\s*=\s*([-0-9.eE]+)", blk).group(1)) for n in names}
    mct["fiducial"] = float(re.search(r"fiducialInverseCrossingTime\s*=\s*([-0-9.eE]+)", blk).group(1))
    mct["gamma"] = 5.0 / 3.0
    mct["source"] = "src/hydro/hydro_cuda_tests.cu:116-142"
    return {"calc_dt_3d": calc, "hydro_inverse_crossing_time": ict, "mhd_inverse_crossing_time": mct}


def hllc_cases(src_dir: Path) -> dict:
    """The HLLC known answer: a Sod high-pressure state against itself (primitive density,
    pressure, velocities and gamma as the test writes them) and its fiducial flux."""
    s = re.sub(r"//[^\n]*", "", (src_dir / "riemann_solvers/hllc_cuda_tests.cu").read_text())
    cases = []
    for name, body in _test_bodies(s, "tHYDROCalculateHLLCFluxesCUDA").items():
        consts = {}
        for c in re.finditer(r"Real\s+const\s+(\w+)\s*=\s*([^;{]+);", body):
            consts[c.group(1)] = _cpp_value(c.group(2), consts)
        fid, _ = initializer(body, "fiducialFluxes")
        prim = [consts[k] for k in ("density", "velocityX", "velocityY", "velocityZ", "pressure")]
        cases.append({"test": name, "left": prim, "right": prim, "gamma": consts["gamma"],
                      "fiducial": [float(v) for v in fid]})
    return {"cases": cases, "source": "src/riemann_solvers/hllc_cuda_tests.cu:152-176"}


def _matching(s: str, i: int) -> int:
    """Index of the brace that closes the one at s[i]."""
    depth = 0
    for j in range(i, len(s)):
        depth += (s[j] == "{") - (s[j] == "}")
        if depth == 0:
            return j
    raise ValueError("unbalanced braces")


def _cpp_value(expr: str, consts: dict) -> float:
    """A C++ arithmetic literal expression of the test sources (numbers, named constants,
    std::sqrt, M_PI) as a float."""
    e = " ".join(expr.split()).replace("std::sqrt", "math.sqrt").replace("std::pow", "math.pow").replace("M_PI", "math.pi")
    e = re.sub(r"(?<![\w.])(\d+)\.(?![\d\w])", r"\1.0", e)  # "2." -> "2.0"
    return float(eval(e, {"math": math, "__builtins__": {}}, dict(consts)))


def hlld_cases(src_dir: Path) -> dict:
    """The known-answer flux tests of mhd::Calculate_HLLD_Fluxes_CUDA: per case the left and
    right primitive states (density, vx, vy, vz, pressure, Bx, By, Bz), gamma, the interface
    directions the test loops over, and the fiducial flux (density, momenta, energy, Bx, By,
    Bz).  Cases whose states the test edits in place are kept only for the edits recognised
    here (Bx sign flips); the rest are counted as skipped."""
    s = re.sub(r"//[^\n]*", "", (src_dir / "riemann_solvers/hlld_cuda_tests.cu").read_text())
    cases, skipped = [], 0
    for m in re.finditer(r"TEST_F\(tMHDCalculateHLLDFluxesCUDA,\s*(\w+)\)", s):
        i = s.index("{", m.end())
        body = s[i:_matching(s, i) + 1]
        consts = {}
        for c in re.finditer(r"Real\s+const\s+(\w+)\s*=\s*([^;{]+);", body):
            try:
                consts[c.group(1)] = _cpp_value(c.group(2), consts)
            except Exception:
                pass
        states = {}
        for st in re.finditer(r"(\w+)\s*=\s*Primitive_2_Conserved\(\s*\{([^}]*)\}", body):
            states[st.group(1)] = [_cpp_value(x, consts) for x in st.group(2).split(",")]
        dirs = [0, 1, 2] if re.search(r"for\s*\(size_t direction", body) else [0]
        for f in re.finditer(r"fiducialFlux\s*\{", body):
            k = body.index("{", f.start())
            k2 = _matching(body, k)
            fid = [_cpp_value(x, consts) for x in body[k + 1:k2].split(",")]
            call = re.search(r"Compute_Fluxes\(\s*(\w+)\s*,\s*(\w+)\s*,\s*gamma", body[k2:])
            if not call:
                skipped += 1
                continue
            between = body[k2:k2 + call.start()]
            left, right = call.group(1), call.group(2)
            flips = {}
            for nm in (left, right):
                base = re.search(rf"\b{nm}\s*=\s*(\w+)\s*[,;]", between)
                if base and re.search(rf"{nm}\[5\]\s*=\s*-{nm}\[5\]", between):
                    flips[nm] = base.group(1)
            def state(nm):
                if nm in flips:
                    v = list(states[flips[nm]])
                    v[5] = -v[5]
                    return v
                return states.get(nm)
            L, R = state(left), state(right)
            edits = re.sub(r"(std::vector<Real>\s+const\s+scalarFlux\s*\{[^}]*\};|Real\s+thermalEnergyFlux\s*=[^;]*;)",
                           "", between)
            edits = re.sub(r"std::vector<Real>\s+(\w+)\s*=\s*(\w+)\s*,\s*(\w+)\s*=\s*(\w+)\s*;", "", edits)
            edits = re.sub(r"\w+\[5\]\s*=\s*-\w+\[5\]\s*;", "", edits)
            edits = re.sub(r"^\s*\}\s*;|std::vector<Real>\s+const\s+testFluxes\s*=\s*$", "", edits.strip()).strip()
            if L is None or R is None or len(fid) != 8 or edits:
                skipped += 1
                continue
            cases.append({"test": m.group(1), "gamma": consts["gamma"], "left": L, "right": R, "directions": dirs,
                          "fiducial": fid})
    return {"cases": cases, "skipped": skipped, "rule": {"abs": 2.7e-15, "ulps": 7},
            "source": "src/riemann_solvers/hlld_cuda_tests.cu:30-1875"}


def _test_bodies(s: str, suite: str) -> dict:
    """{test name: body} of the TEST_F / TEST blocks of one suite, comments removed."""
    s = re.sub(r"//[^\n]*", "", s)
    out = {}
    for m in re.finditer(rf"TEST(?:_F|_P)?\({suite},\s*(\w+)\)", s):
        i = s.index("{", m.end())
        out[m.group(1)] = s[i:_matching(s, i) + 1]
    return out


def _at_assignments(body: str, name: str) -> dict:
    return {k: float(v) for k, v in re.findall(rf"{name}\.at\((\d+)\)\s*=\s*([-+0-9.eE]+)\s*;", body)}


def _fixture_value(s: str, name: str) -> float:
    return float(re.search(rf"\b{name}\s*=\s*([-+0-9.eE]+)\s*[,;]", s).group(1))


def mhd_unit_cases(src_dir: Path) -> dict:
    """Known answers of the MHD kernels: the CT electric fields and the face-field update on
    iota-filled grids (every array holds 0, 1, 2, ... continuing from the previous one), the CT
    slope at the centre of a 5^3 grid and the maximum divergence of a 104^3 grid, both filled
    from std::mt19937(1) draws.  Every entry not named in `fiducial` keeps its -999 fill."""
    ct_src = (src_dir / "mhd/ct_electric_fields_tests.cu").read_text()
    ct = []
    for name, body in _test_bodies(ct_src, "tMHDCalculateCTElectricFields").items():
        if re.search(r"fluxX\.at\(i\)\s*=\s*-fluxX\.at\(i\)", body):
            edit = "negate_first_field"
        elif re.search(r"fluxX\.at\(i\)\s*=\s*0(\.0*)?\s*;", body):
            edit = "zero_first_field"
        elif "fluxX.at(i)" in body:
            continue
        else:
            edit = "none"
        ct.append({"test": name, "edit": edit, "fiducial": _at_assignments(body, "fiducialData")})
    n_ct = int(_fixture_value(ct_src, "size_t const nx"))
    slope_body = _test_bodies(ct_src, "tMHDCTSlope")["CorrectInputExpectCorrectOutput"]
    fid, _ = initializer(slope_body, "fiducial_data")
    calls = re.findall(r"_ctSlope\(flux\.data\(\),\s*conserved\.data\(\),\s*([-\d]+),\s*([-\d]+),\s*([-\d]+),"
                       r"\s*([-\d]+),\s*([-\d]+),\s*([-\d]+),", slope_body)
    rng = re.search(r"doubleRand\(([-\d.]+),\s*([-\d.]+)\)", slope_body)
    up_src = (src_dir / "mhd/magnetic_update_tests.cu").read_text()
    up_body = _test_bodies(up_src, "tMHDUpdateMagneticField3D")["CorrectInputExpectCorrectOutput"]
    div_src = (src_dir / "mhd/magnetic_divergence_tests.cu").read_text()
    div_body = _test_bodies(div_src, "tMHDGrid3DcheckMagneticDivergence")["CorrectInputExpectCorrectOutput"]
    div_rng = re.search(r"doubleRand\(([-\d.]+),\s*([-\d.]+)\)", div_body)
    scale = float(re.search(r"doubleRand\(prng\)\s*/\s*([-+0-9.eE]+)", div_body).group(1))
    fid_div = re.search(r"fiducialDivergence\s*=\s*([-+0-9.eE]+)\s*/\s*([-+0-9.eE]+)", div_body)
    return {
        "rule": {"abs": 1e-14, "ulps": 4},
        "ct_electric_fields": {"n": n_ct, "n_fields": 8, "n_flux_fields": 7, "cases": ct,
                               "source": "src/mhd/ct_electric_fields_tests.cu:35-178"},
        "ct_slope": {"n": int(re.search(r"size_t const nx\s*=\s*(\d+)", slope_body).group(1)), "n_fields": 8,
                     "seed": int(re.search(r"std::mt19937 prng\((\d+)\)", slope_body).group(1)),
                     "range": [float(rng.group(1)), float(rng.group(2))],
                     "calls": [[int(v) for v in c] for c in calls], "fiducial": [float(v) for v in fid],
                     "source": "src/mhd/ct_electric_fields_tests.cu:183-272"},
        "update_magnetic": {"n": int(_fixture_value(up_src, "size_t const nx")), "n_fields": 8,
                            "dt": _fixture_value(up_src, "Real const dt"), "dx": _fixture_value(up_src, "dx"),
                            "fiducial": _at_assignments(up_body, "fiducialData"),
                            "source": "src/mhd/magnetic_update_tests.cu:28-124"},
        "max_divergence": {"n_real": int(re.search(r"gridSize\s*=\s*(\d+)", div_body).group(1)),
                           "n_ghost": int(re.search(r"n_ghost\s*=\s*(\d+)", div_body).group(1)),
                           "n_fields": int(re.search(r"n_fields\s*=\s*(\d+)", div_body).group(1)),
                           "dx": float(re.search(r"G\.H\.dx\s*=\s*([-+0-9.eE]+)", div_body).group(1)),
                           "seed": int(re.search(r"std::mt19937 prng\((\d+)\)", div_body).group(1)),
                           "range": [float(div_rng.group(1)), float(div_rng.group(2))], "scale": scale,
                           "fiducial": float(fid_div.group(1)) / float(fid_div.group(2)),
                           "source": "src/mhd/magnetic_divergence_tests.cu:27-65"},
    }


def _preprocess(src: str, defined: set) -> str:
    """The source with `#ifdef` / `#ifndef` / `#if defined(X)` / `#elif defined(X)` / `#else` /
    `#endif` branches resolved for the given macros (other directives dropped)."""
    def cond_of(expr: str) -> bool:
        m = re.fullmatch(r"\s*(?:defined\s*\(\s*(\w+)\s*\)|defined\s+(\w+)|(\w+))\s*", expr)
        return bool(m) and (m.group(1) or m.group(2) or m.group(3)) in defined

    out, stack = [], []  # entries: [this branch active, some branch taken]
    for line in src.splitlines():
        t = line.strip()
        m = re.match(r"#\s*(ifdef|ifndef)\s+(\w+)", t)
        if m:
            c = (m.group(2) in defined) == (m.group(1) == "ifdef")
            stack.append([c, c])
            continue
        m = re.match(r"#\s*if\s+(.*)", t)
        if m:
            c = cond_of(re.sub(r"//.*", "", m.group(1)))
            stack.append([c, c])
            continue
        m = re.match(r"#\s*elif\s+(.*)", t)
        if m:
            c = not stack[-1][1] and cond_of(re.sub(r"//.*", "", m.group(1)))
            stack[-1] = [c, stack[-1][1] or c]
            continue
        if re.match(r"#\s*else\b", t):
            stack[-1] = [not stack[-1][1], True]
            continue
        if re.match(r"#\s*endif\b", t):
            stack.pop()
            continue
        if t.startswith("#"):
            continue
        if all(c for c, _ in stack):
            out.append(line)
    return "\n".join(out)


def reconstruction_helpers(src_dir: Path) -> dict:
    """The helper unit tests of src/reconstruction/reconstruction_tests.cu that sit on the VL
    path, for the MHD and the hydro build: per test the literal structs it builds
    (reconstruction::Primitive / Characteristic / EigenVecs, in member order), its scalar
    constants, field assignments, fiducial maps and any per-field tolerance it passes."""
    raw = (src_dir / "reconstruction/reconstruction_tests.cu").read_text()
    names = ["tMHDReconstructionPrimitive2Characteristic", "tMHDReconstructionCharacteristic2Primitive",
             "tMHDReconstructionComputeEigenvectors", "tALLReconstructionThreadGuard", "tALLReconstructionLoadData",
             "tALLReconstructionComputeSlope", "tALLReconstructionVanLeerSlope",
             "tALLReconstructionMonotonizeCharacteristicReturnPrimitive", "tALLReconstructionCalcInterfaceLinear",
             "tALLReconstructionWriteData", "tHYDROReconstructionPlmLimitInterfaces"]
    out = {}
    for build, defined in (("mhd", {"MHD"}), ("hydro", set())):
        src = re.sub(r"//[^\n]*", "", _preprocess(raw, defined))
        tests = {}
        for name in names:
            bodies = _test_bodies(src, name)
            if not bodies:
                continue
            body = bodies["CorrectInputExpectCorrectOutput"]
            structs = {m.group(2): [_cpp_value(v, {}) for v in m.group(3).split(",") if v.strip()]
                       for m in re.finditer(r"reconstruction::(?:Primitive|Characteristic|EigenVecs)\s+(const\s+)?(\w+)"
                                            r"\s*\{([^}]*)\}", body)}
            consts = {}
            for m in re.finditer(r"(?:Real|int|size_t)\s+const\s+([^;]+);", body):
                for part in m.group(1).split(","):
                    k, _, v = part.partition("=")
                    try:
                        consts[k.strip().lstrip("&")] = _cpp_value(v, consts)
                    except Exception:
                        pass
            fields = {}
            for m in re.finditer(r"(\w+)\.(\w+)\s*=\s*([-+0-9.eE]+)\s*;", body):
                fields.setdefault(m.group(1), {})[m.group(2)] = float(m.group(3))
            fmap = re.search(r"unordered_map<int,\s*double>\s+\w+\s*=\s*\{(.*?)\};", body, re.S)
            tol = {m.group(1): float(m.group(2)) for m in re.finditer(
                r"Check_Results\(fiducial_\w+\.(\w+),\s*host_results\.\w+,\s*\"\w+\",\s*([-+0-9.eE]+)\)", body)}
            tests[name] = {"structs": structs, "consts": consts, "fields": fields,
                           "map": {int(a): float(b) for a, b in re.findall(r"\{\s*(\d+)\s*,\s*([-+0-9.eE]+)\s*\}",
                                                                          fmap.group(1))} if fmap else {},
                           "at": _at_assignments(body, "fiducial_vals"), "abs_tolerance": tol}
        out[build] = tests
    out["source"] = "src/reconstruction/reconstruction_tests.cu:51-699"
    return out


def _braces(src: str, name: str):
    """JSON value of the brace initializer that follows `name` (std::nan -> NaN)."""
    m = re.search(rf"\b{re.escape(name)}\s*(=\s*)?\{{", src)
    i = src.index("{", m.start())
    text = src[i:_matching(src, i) + 1]
    text = re.sub(r"std::nan\(\"0\"\)", "NaN", text)
    return braces_to_json(text)


def hlld_internal_cases(src_dir: Path) -> dict:
    """The HLLD-internal unit tests (mhd::internal::*): the shared TestParams (two cases of left
    and right states, star states, fluxes, speeds, the star total pressure and the normal field)
    and per test its fiducial vectors and the per-field absolute tolerances it passes."""
    s = re.sub(r"//[^\n]*", "", (src_dir / "riemann_solvers/hlld_cuda_tests.cu").read_text())
    i = s.index("struct TestParams")
    tp_src = s[i:_matching(s, s.index("{", i)) + 1]
    params = {k: _braces(tp_src, k) for k in ("magneticX", "stateLVec", "stateRVec", "starStateLVec", "starStateRVec",
                                              "totalPressureStar", "DoubleStarStateVec", "flux", "starFlux", "speed")}
    params["gamma"] = _cpp_value(re.search(r"double const gamma\s*=\s*([^;]+);", tp_src).group(1), {})
    tests = {}
    for m in re.finditer(r"TEST\((tMHDHlldInternal\w+),\s*(\w+)\)", s):
        j = s.index("{", m.end())
        body = s[j:_matching(s, j) + 1]
        fid = {}
        for f in re.finditer(r"std::vector<[\w:]+>\s+(?:const\s+)?(fiducial\w+)\s*\{", body):
            fid[f.group(1)] = _braces(body, f.group(1))
        tol = {t.group(1): float(t.group(2)) for t in re.finditer(
            r"Check_Results\(fiducial\w+(?:\[i\]|\.at\(i\))\.(\w+),\s*test\w+\.\w+,[^;]*?,\s*([-+0-9.eE]+)\)", body)}
        mult = re.search(r"totalPressureStarMultiplier\s*=\s*([-+0-9.eE]+)", body)
        entry = {"fiducial": fid, "abs_tolerance": tol,
                 "multiplier": float(mult.group(1)) if mult else None}
        if m.group(1) == "tMHDHlldInternalReturnFluxes":
            entry["flux"] = _braces(body, "inputFlux")
            entry["state"] = _braces(body, "inputState")
            entry["dummy"] = float(re.search(r"dummyValue\s*=\s*([-+0-9.eE]+)", body).group(1))
        if m.group(1) == "tMHDHlldInternalLoadState":
            entry["n_cells"] = int(re.search(r"n_cells\s*=\s*(\d+)", body).group(1))
        tests[m.group(1) + "." + m.group(2)] = entry
    return {"params": params, "tests": tests, "source": "src/riemann_solvers/hlld_cuda_tests.cu:1811-2400"}


def _vectors(body: str) -> dict:
    """Every `std::vector<double> [const] name{...}` of a test body, by name."""
    return {m.group(1): [_cpp_value(v, {}) for v in m.group(2).split(",") if v.strip()]
            for m in re.finditer(r"std::vector<double>\s+(?:const\s+)?(\w+)\s*\{([^}]*)\}", body)}


def utility_cases(src_dir: Path) -> dict:
    """The unit tests of the hydro and MHD utility functions that the VL step calls (for the MHD
    and the hydro build where the fiducials differ): the shared TestParams vectors and per test
    its fiducial vector, its multipliers (`coef` scalars or vectors) and the first case it loops
    from."""
    out = {}
    for key, rel in (("hydro_utilities", "utils/hydro_utilities_tests.cpp"),
                     ("mhd_utilities", "utils/mhd_utilities_tests.cu")):
        raw = (src_dir / rel).read_text()
        for build, defined in (("mhd", {"MHD"}), ("hydro", set())):
            src = re.sub(r"//[^\n]*", "", _preprocess(raw, defined))
            i = src.index("struct TestParams")
            params = _vectors(src[i:_matching(src, src.index("{", i)) + 1])
            params["gamma"] = 5.0 / 3.0
            tests = {}
            for m in re.finditer(r"TEST\((\w+),\s*(\w+)\)", src):
                j = src.index("{", m.end())
                body = src[j:_matching(src, j) + 1]
                coef = re.search(r"double const coef\s*=\s*([-+0-9.eE]+)", body)
                start = re.search(r"for \(size_t i = (\d+);", body)
                consts = {}
                for c in re.finditer(r"(?:double|Real|size_t)\s+const\s+([^;]+);", body):
                    for part in c.group(1).split(","):
                        k, _, v = part.partition("=")
                        try:
                            consts[k.strip()] = _cpp_value(v, consts)
                        except Exception:
                            pass
                tests[m.group(1) + "." + m.group(2)] = {
                    "vectors": _vectors(body), "coef": float(coef.group(1)) if coef else None,
                    "start": int(start.group(1)) if start else 0, "consts": consts}
            out.setdefault(key, {})[build] = {"params": params, "tests": tests}
        out[key]["source"] = "src/" + rel
    return out


def hydro_system_cases(src_dir: Path) -> dict:
    """The analytic hydro system tests (src/system_tests/hydro_system_tests.cpp): the linear
    sound and contact waves on 64 x 32 x 32 cells run for one wave period (expected step count,
    per-field L1 bound, bound on the norm of the L1 vector and on the maximum error, per
    reconstruction), and the 3D sound wave at t = 0.05 against the analytic sine (settings from
    its input file)."""
    raw = (src_dir / "system_tests/hydro_system_tests.cpp").read_text()
    out = {"linear_waves": {}, "source": "src/system_tests/hydro_system_tests.cpp:99-306"}
    for recon in ("PCM", "PLMC", "PPMC", "PLMP", "PPMP"):
        src = re.sub(r"//[^\n]*", "", _preprocess(raw, {recon}))
        allowed = {k: float(v) for k, v in re.findall(r"double static constexpr (allowedL1Error|allowedError)\s*=\s*"
                                                      r"([-+0-9.eE]+)", src)}
        i = src.index("void Set_Launch_Params")
        body = src[i:_matching(src, src.index("{", i)) + 1]
        setup = {k: _cpp_value(v, {}) for k, v in re.findall(r"(?:size_t|double) const (N|domain|gamma)\s*=\s*([^;]+);",
                                                            body)}
        waves = {}
        for name, tb in _test_bodies(src, "tHYDROtMHDSYSTEMLinearWavesParameterizedMpi").items():
            consts = {}
            for c in re.finditer(r"(?:double|int) const (\w+)\s*=\s*([^;]+);", tb):
                consts[c.group(1)] = _cpp_value(c.group(2), consts)
            call = re.search(r"runL1ErrorTest\(([^,]+),\s*([^)]+)\)", tb)
            scale = lambda e: _cpp_value(e, allowed)
            waves[name] = {"wave_speed": consts["waveSpeed"], "n_steps": int(consts["numTimeSteps"]),
                           "eigen": {k[len("rEigenVec_"):]: v for k, v in consts.items() if k.startswith("rEigenVec_")},
                           "vx": consts.get("velocityX", 0.0),
                           "max_l1": scale(call.group(1)), "max_error": scale(call.group(2))}
        out["linear_waves"][recon] = {"setup": setup, "waves": waves}
    src = re.sub(r"//[^\n]*", "", _preprocess(raw, set()))
    tb = _test_bodies(src, "tHYDROtMHDSYSTEMSoundWave3D")["CorrectInputExpectCorrectOutput"]
    consts = {}
    for c in re.finditer(r"double (?:const )?(\w+)\s*=\s*([^;]+);", tb):
        try:
            consts[c.group(1)] = _cpp_value(c.group(2), consts)
        except Exception:
            pass
    settings = {}
    for line in (src_dir / "system_tests/input_files/tHYDROtMHDSYSTEMSoundWave3D_CorrectInputExpectCorrectOutput.txt"
                 ).read_text().splitlines():
        k, eq, v = line.partition("=")
        if eq and not line.startswith("#"):
            try:
                settings[k.strip()] = float(v.strip().strip("'"))
            except ValueError:
                pass
    # the reference loosens the tolerance per reconstruction in its MHD build ("about the error
    # between PCM and PPMP in hydro"); its hydro build (PLMC) keeps the plain one
    pcm = re.sub(r"//[^\n]*", "", _preprocess(raw, {"MHD", "PCM"}))
    pcm_body = _test_bodies(pcm, "tHYDROtMHDSYSTEMSoundWave3D")["CorrectInputExpectCorrectOutput"]
    pcm_tol = float(re.findall(r"tolerance\s*=\s*([-+0-9.eE]+)\s*;", pcm_body)[-1])
    out["sound_wave_3d"] = {"time": consts["time"], "amplitude": consts["amplitude"],
                            "tolerance": {"PCM": pcm_tol, "PLMC": consts["tolerance"], "PPMC": consts["tolerance"]},
                            "settings": settings, "source": "src/system_tests/hydro_system_tests.cpp:99-132"}
    return out


def mhd_system_cases(src_dir: Path) -> dict:
    """The MHD linear-wave system tests at angles (src/system_tests/mhd_system_tests.cpp:30-541):
    fast, slow and Alfven waves in both directions and the contact wave, each along x, y and z
    (the instantiated pitch / yaw / domain / direction tuples), with the step count per
    direction and the L1 / maximum-error bounds per reconstruction; and the N = 16 runs whose
    L1 norm must be four times the N = 32 one (second-order convergence)."""
    raw = (src_dir / "system_tests/mhd_system_tests.cpp").read_text()
    base = re.sub(r"//[^\n]*", "", _preprocess(raw, {"MHD", "PLMC"}))
    inst = base[base.index("INSTANTIATE_TEST_SUITE_P(, tMHDSYSTEMLinearWavesParameterizedAngle"):]
    inst = inst[:inst.index(";")]
    angles = [[_cpp_value(v, {}) for v in t.split(",")]
              for t in re.findall(r"std::make_tuple\(([^)]*)\)", inst)]
    tests = {}
    for recon in ("PCM", "PLMC", "PPMC"):
        src = re.sub(r"//[^\n]*", "", _preprocess(raw, {"MHD", recon}))
        for name, tb in _test_bodies(src, "tMHDSYSTEMLinearWavesParameterizedAngle").items():
            consts = {}
            for c in re.finditer(r"double const (\w+)\s*=\s*([^;]+);", tb):
                try:
                    consts[c.group(1)] = _cpp_value(c.group(2), consts)
                except NameError:  # values read back from the runner (the L2 norms)
                    pass
            call = re.search(r"Set_Launch_Params\(([^;]*)\);", tb).group(1)
            args = [a.strip() for a in call.split(",")]
            entry = tests.setdefault(name, {
                "wave_speed": consts["waveSpeed"],
                "n_steps": [int(v) for v in _braces(tb, "numTimeSteps")],
                "eigen": {k[len("rEigenVec_"):]: v for k, v in consts.items() if k.startswith("rEigenVec_")},
                "vx": _cpp_value(args[13], consts) if len(args) > 13 else 0.0,
                "N": int(args[14]) if len(args) > 14 else 32, "bounds": {}})
            b = re.search(r"runL1ErrorTest\(([^,]+),\s*([^)]+)\)", tb)
            entry["bounds"][recon] = [_cpp_value(b.group(1), {}), _cpp_value(b.group(2), {})]
            conv = re.search(r"high_res_l2norms\[\"(\w+)_\"", tb)
            if conv and "Convergence" in name:
                tol = re.search(r"Check_Results\(\s*([-+0-9.eE]+),[^;]*,\s*\"\",\s*([-+0-9.eE]+)\)", tb)
                entry["convergence"] = {"of": conv.group(1), "ratio": float(tol.group(1)), "tolerance": float(tol.group(2))}
            elif conv:
                entry["key"] = conv.group(1)
    return {"angles": angles, "tests": tests, "B": [1.0, 1.5, 0.0], "gamma": 5.0 / 3.0, "amplitude": 1e-6,
            "source": "src/system_tests/mhd_system_tests.cpp:30-541"}


def _settings(path: Path) -> dict:
    out = {}
    for line in path.read_text().splitlines():
        k, eq, v = line.partition("=")
        if eq and not line.lstrip().startswith("#"):
            try:
                out[k.strip()] = float(v.strip().strip("'"))
            except ValueError:
                pass
    return out


def constant_state_cases(src_dir: Path) -> dict:
    """The constant-state system tests: the settings of their input files and, for the hydro
    one, the analytic values the test checks (hydro_system_tests.cpp:84-97).  The MHD ones
    (mhd_system_tests.cpp:710-722) compare with data files absent here; a constant state is
    their only possible answer."""
    inp = src_dir / "system_tests/input_files"
    raw = re.sub(r"//[^\n]*", "", (src_dir / "system_tests/hydro_system_tests.cpp").read_text())
    body = _test_bodies(raw, "tHYDROtMHDSYSTEMConstant")["CorrectInputExpectCorrectOutput"]
    expect = {k: float(v) for k, v in re.findall(r"analyticConstant\(testObject,\s*\"(\w+)\",\s*([-+0-9.eE]+)\)", body)}
    return {
        "hydro": {"settings": _settings(inp / "tHYDROtMHDSYSTEMConstant_CorrectInputExpectCorrectOutput.txt"),
                  "expect": expect, "abs_tolerance": 5.0e-12},
        "mhd_field": {"settings": _settings(
            inp / "tMHDSYSTEMParameterizedMpi_ConstantWithMagneticFieldCorrectInputExpectCorrectOutput.txt")},
        "mhd_zero_field": {"settings": _settings(
            inp / "tMHDSYSTEMParameterizedMpi_ConstantWithZeroMagneticFieldCorrectInputExpectCorrectOutput.txt")},
        "source": "src/system_tests/hydro_system_tests.cpp:84-97, mhd_system_tests.cpp:710-722",
    }


def main() -> None:
    root = Path(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CHOLLA_REFERENCE", Path(__file__).resolve().parents[3] / "reference"))
    src = root / "src"
    data = {
        "note": "golden vectors read from the reference's unit tests by extract_reference_fiducials.py",
        "ppmc_vl": ppmc_vl(src),
        "plmc": plmc(src),
        "ppm_single_variable": ppm_single_variable(src),
        "reconstruction_helpers": reconstruction_helpers(src),
        "dt": dt_tests(src),
        "hllc": hllc_cases(src),
        "hlld": hlld_cases(src),
        "hlld_internal": hlld_internal_cases(src),
        "utilities": utility_cases(src),
        "hydro_system": hydro_system_cases(src),
        "mhd_system": mhd_system_cases(src),
        "constant_states": constant_state_cases(src),
        "mhd_unit": mhd_unit_cases(src),
    }
    out = HERE / "reference_fiducials.json"
    out.write_text(json.dumps(data, indent=1))
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
