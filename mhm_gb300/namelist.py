"""mHM's Fortran namelists (mhm.nml, mhm_parameter.nml) and the run
configuration the drop-in takes from them.

`read` parses namelist text: groups `&name ... /`, `!` comments, scalars,
arrays with index ranges (`evap_coeff(1:12) = ...`, `soil_depth(1) = 200`),
two-dimensional indexes (`gauge_id(2,1) = 398`, `GeoParam(3,:) = ...`),
derived-type components (`eval_per(1)%ystart = 1990`), values continued over
lines, `r*value` repeats, quoted strings, logicals and Fortran reals with
`d` exponents.  Keys are case-insensitive, as in Fortran.

`run_config` takes from mhm.nml the subset the drop-in needs -- process
cases, time step, soil horizons, pan-evaporation and day/night tables, the
sealed fraction of city areas, periods, resolutions, evaluation and inflow
gauges, land-cover scenes (the keys read by src/common/mo_common_read_config.f90,
src/mHM/mo_mhm_read_config.f90, src/MPR/mo_mpr_read_config.f90 and
src/mRM/mo_mrm_read_config.f90) -- and `gamma` lays out the global
parameter vector from mhm_parameter.nml: the `value` column of the process
blocks in processMatrix order (src/MPR/mo_mpr_read_config.f90:390-990).
`to_json` / `from_json` write and read a namelist as JSON with the same
groups and keys (group -> key -> value, arrays as index -> value maps), a
1:1 image of the text.
"""
from __future__ import annotations

import json
import re
from dataclasses import dataclass, field
from pathlib import Path

_NAME = r"[A-Za-z_][A-Za-z0-9_]*"
_ASSIGN = re.compile(rf"({_NAME})\s*(\([^)]*\))?\s*(%\s*{_NAME})?\s*=")


@dataclass
class Assignment:
    key: str             # lower case
    index: str | None    # the text inside the parentheses, blanks removed, or None
    component: str | None  # derived-type component after '%', lower case
    values: list


def _strip_comment(line: str) -> str:
    out, quote = [], None
    for ch in line:
        if quote:
            if ch == quote:
                quote = None
        elif ch in "'\"":
            quote = ch
        elif ch == "!":
            break
        out.append(ch)
    return "".join(out)


def _split_values(text: str) -> list[str]:
    toks, cur, quote = [], [], None
    for ch in text:
        if quote:
            cur.append(ch)
            if ch == quote:
                quote = None
            continue
        if ch in "'\"":
            quote = ch
            cur.append(ch)
        elif ch in ", \t\n":
            if cur:
                toks.append("".join(cur))
                cur = []
        else:
            cur.append(ch)
    if cur:
        toks.append("".join(cur))
    return toks


def _value(tok: str):
    t = tok.strip()
    if len(t) >= 2 and t[0] in "'\"" and t[-1] == t[0]:
        return t[1:-1].replace(t[0] * 2, t[0])
    low = t.lower()
    if low in (".true.", ".t.", "t", "true"):
        return True
    if low in (".false.", ".f.", "f", "false"):
        return False
    if re.fullmatch(r"[+-]?\d+", t):
        return int(t)
    try:
        return float(low.replace("d", "e"))
    except ValueError as e:
        raise ValueError(f"namelist value {tok!r} not understood") from e


def _values(text: str) -> list:
    out = []
    for tok in _split_values(text):
        m = re.fullmatch(r"(\d+)\*(.+)", tok)
        if m and not tok.startswith(("'", '"')):
            out.extend([_value(m.group(2))] * int(m.group(1)))
        else:
            out.append(_value(tok))
    return out


def read(source) -> dict[str, list[Assignment]]:
    """Groups of a namelist file (a path) or text: {group (lower case): [assignments in order]}."""
    text = Path(source).read_text() if isinstance(source, Path) or (
        isinstance(source, str) and "\n" not in source and Path(source).exists()) else str(source)
    lines = [_strip_comment(ln) for ln in text.splitlines()]
    groups: dict[str, list[Assignment]] = {}
    body: list[str] | None = None
    name = None
    for ln in lines + [""]:
        s = ln.strip()
        if body is None:
            m = re.match(rf"&({_NAME})(.*)$", s)
            if m:
                name = m.group(1).lower()
                rest = m.group(2).strip()
                body = []
                if rest.endswith("/"):
                    body.append(rest[:-1])
                    groups[name] = _assignments(" ".join(body))
                    body = None
                elif rest:
                    body.append(rest)
            continue
        if s == "/" or s.endswith("/") and not s.endswith("//") and _closes(s):
            body.append(s[:-1])
            groups[name] = _assignments("\n".join(body))
            body = None
        else:
            body.append(ln)
    if body is not None:
        raise ValueError(f"namelist group &{name} not closed with '/'")
    return groups


def _closes(s: str) -> bool:
    """a trailing '/' outside quotes ends the group"""
    quote = None
    for ch in s[:-1]:
        if quote:
            if ch == quote:
                quote = None
        elif ch in "'\"":
            quote = ch
    return quote is None


def _assignments(body: str) -> list[Assignment]:
    out = []
    matches = list(_ASSIGN.finditer(body))
    # assignments start where a key is followed by '=' outside a string value
    starts = [m for m in matches if not _inside_quotes(body, m.start())]
    for i, m in enumerate(starts):
        end = starts[i + 1].start() if i + 1 < len(starts) else len(body)
        idx = m.group(2)
        comp = m.group(3)
        out.append(Assignment(m.group(1).lower(), re.sub(r"\s+", "", idx[1:-1]) if idx else None,
                              comp.replace("%", "").strip().lower() if comp else None,
                              _values(body[m.end():end])))
    return out


def _inside_quotes(text: str, pos: int) -> bool:
    quote = None
    for ch in text[:pos]:
        if quote:
            if ch == quote:
                quote = None
        elif ch in "'\"":
            quote = ch
    return quote is not None


# ---- arrays from assignments ----

def _range(spec: str) -> list[int]:
    if ":" in spec:
        a, b = spec.split(":")
        return list(range(int(a), int(b) + 1))
    return [int(spec)]


def array(groups, group: str, key: str, component: str | None = None) -> dict:
    """{index tuple: value} of every element assigned to key (1-based Fortran
    indexes; a scalar assignment has the index ())."""
    out = {}
    for a in groups.get(group.lower(), []):
        if a.key != key.lower() or a.component != (component.lower() if component else None):
            continue
        if a.index is None:
            if len(a.values) == 1:
                out[()] = a.values[0]
            else:
                for i, v in enumerate(a.values):
                    out[(i + 1,)] = v
            continue
        dims = a.index.split(",")
        if len(dims) == 1:
            idx = _range(dims[0])
            if len(a.values) == 1 and len(idx) > 1:
                raise ValueError(f"{key}({a.index}): one value for {len(idx)} elements")
            for i, v in zip(idx, a.values):
                out[(i,)] = v
        else:
            # fill the first open dimension fastest (Fortran order); a ':'
            # alone is the whole extent of the values given
            ranges = [list(range(1, len(a.values) + 1)) if d == ":" else _range(d) for d in dims]
            cells = [()]
            for r in reversed(ranges):
                cells = [(i,) + c for i in r for c in cells]
            cells = sorted(cells, key=lambda c: tuple(reversed(c)))
            for c, v in zip(cells, a.values):
                out[c] = v
    return out


def get(groups, group: str, key: str, default=None, component: str | None = None):
    """A scalar, or the 1-D array (list) of a key whose indexes are 1..n."""
    a = array(groups, group, key, component)
    if not a:
        return default
    if () in a:
        return a[()]
    if all(len(k) == 1 for k in a):
        n = max(k[0] for k in a)
        return [a.get((i,), default) for i in range(1, n + 1)]
    return a


# ---- the drop-in's run configuration ----

PET_BLOCK = {-1: "petminus1", 0: "pet0", 1: "pet1", 2: "pet2", 3: "pet3"}


@dataclass
class RunConfig:
    process_case: list            # processCase(1:10)
    timestep: int                 # hours
    n_soil_horizons: int
    soil_depth: list              # mm, horizons 1 .. n-1 (the last reaches the soil's depth)
    tillage_depth: float
    evap_coeff: list              # [12]
    fnight_prec: list
    fnight_pet: list
    fnight_temp: list
    frac_sealed_city_area: float
    n_domains: int = 1
    resolution_hydrology: list = field(default_factory=list)
    resolution_routing: list = field(default_factory=list)
    warming_days: list = field(default_factory=list)
    eval_per: list = field(default_factory=list)          # per domain: (ystart, mstart, dstart, yend, mend, dend)
    gauges: list = field(default_factory=list)            # per domain: [gauge ids]
    inflow_gauges: list = field(default_factory=list)     # per domain: [(id, headwater)]
    lcover_years: list = field(default_factory=list)      # [(yearstart, yearend)] per scene

    @property
    def proc_sm(self) -> int:
        return int(self.process_case[2])

    @property
    def proc_pet(self) -> int:
        return int(self.process_case[4])

    @property
    def proc_rout(self) -> int:
        return int(self.process_case[7])

    def fday(self, which: str) -> list:
        """fday_* of the day/night disaggregation: 1 - fnight for prec and PET,
        -fnight for temperature (src/meteo/mo_meteo_handler.f90 disaggregation
        tables)."""
        night = getattr(self, "fnight_" + which)
        return [-x for x in night] if which == "temp" else [1.0 - x for x in night]


def run_config(mhm_nml) -> RunConfig:
    """From an mhm.nml (a path, its text, or groups from `read` / `from_json`)."""
    g = mhm_nml if isinstance(mhm_nml, dict) else read(mhm_nml)
    nd = int(get(g, "mainconfig", "ndomains", 1))

    def per_domain(group, key, comp=None):
        v = get(g, group, key, None, comp)
        if v is None:
            return []
        return v if isinstance(v, list) else [v]

    eval_per = []
    for d in range(1, nd + 1):
        eval_per.append(tuple(int(array(g, "time_periods", "eval_per", c).get((d,), 0))
                              for c in ("ystart", "mstart", "dstart", "yend", "mend", "dend")))
    ids = array(g, "evaluation_gauges", "gauge_id")
    n_g = per_domain("evaluation_gauges", "nogauges_domain")
    gauges = [[ids[(d, i)] for i in range(1, int(n_g[d - 1]) + 1)] if d <= len(n_g) else []
              for d in range(1, nd + 1)]
    in_ids = array(g, "inflow_gauges", "inflowgauge_id")
    in_hw = array(g, "inflow_gauges", "inflowgauge_headwater")
    n_in = per_domain("inflow_gauges", "noinflowgauges_domain")
    inflow = [[(in_ids[(d, i)], bool(in_hw.get((d, i), False))) for i in range(1, int(n_in[d - 1]) + 1)]
              if d <= len(n_in) else [] for d in range(1, nd + 1)]
    ys = per_domain("lcover", "lcoveryearstart")
    ye = per_domain("lcover", "lcoveryearend")
    return RunConfig(
        process_case=[int(x) for x in get(g, "processselection", "processcase")],
        timestep=int(get(g, "mainconfig_mhm_mrm", "timestep")),
        n_soil_horizons=int(get(g, "soildata", "nsoilhorizons_mhm")),
        soil_depth=[float(x) for x in per_domain("soildata", "soil_depth")],
        tillage_depth=float(get(g, "soildata", "tillagedepth")),
        evap_coeff=[float(x) for x in get(g, "panevapo", "evap_coeff")],
        fnight_prec=[float(x) for x in get(g, "nightdayratio", "fnight_prec")],
        fnight_pet=[float(x) for x in get(g, "nightdayratio", "fnight_pet")],
        fnight_temp=[float(x) for x in get(g, "nightdayratio", "fnight_temp")],
        frac_sealed_city_area=float(get(g, "lcover_mpr", "fracsealed_cityarea")),
        n_domains=nd,
        resolution_hydrology=[float(x) for x in per_domain("mainconfig", "resolution_hydrology")],
        resolution_routing=[float(x) for x in per_domain("mainconfig_mhm_mrm", "resolution_routing")],
        warming_days=[int(x) for x in per_domain("time_periods", "warming_days")],
        eval_per=eval_per, gauges=gauges, inflow_gauges=inflow,
        lcover_years=list(zip([int(x) for x in ys], [int(x) for x in ye])))


def gamma(parameter_nml, proc_sm: int, proc_pet: int, proc_rout: int, column: int = 2) -> list[float]:
    """The global parameter vector from mhm_parameter.nml: column 2 (`value`)
    of every row of the process blocks in processMatrix order (column 0 and 1
    give the lower and upper bounds, 3 the optimisation flag)."""
    g = parameter_nml if isinstance(parameter_nml, dict) else read(parameter_nml)
    blocks = ["interception1", "snow1", f"soilmoisture{proc_sm}", "directrunoff1", PET_BLOCK[proc_pet],
              "interflow1", "percolation1"]
    if proc_rout:
        blocks.append(f"routing{proc_rout}")
    blocks.append("geoparameter")
    out = []
    for b in blocks:
        if b not in g:
            raise ValueError(f"parameter namelist has no block &{b}")
        for a in g[b]:
            out.append(float(a.values[column]))
    return out


# ---- JSON image of a namelist ----

def to_json(groups) -> str:
    """{group: {key[%component]: value or {"i[,j]": value}}} -- the namelist's
    groups and keys, arrays as index -> value maps."""
    out = {}
    for name, assigns in groups.items():
        grp = out.setdefault(name, {})
        keys = []
        for a in assigns:
            k = (a.key, a.component)
            if k not in keys:
                keys.append(k)
        for key, comp in keys:
            arr = array(groups, name, key, comp)
            jk = key + (f"%{comp}" if comp else "")
            grp[jk] = arr[()] if list(arr) == [()] else {",".join(map(str, i)): v for i, v in arr.items()}
    return json.dumps(out, indent=1, sort_keys=True)


def from_json(text: str) -> dict[str, list[Assignment]]:
    """The groups of a JSON image (to_json), as `read` returns them."""
    data = json.loads(text)
    groups = {}
    for name, keys in data.items():
        assigns = []
        for jk, v in keys.items():
            key, _, comp = jk.partition("%")
            if isinstance(v, dict):
                for idx, x in v.items():
                    assigns.append(Assignment(key, idx, comp or None, [x]))
            else:
                assigns.append(Assignment(key, None, comp or None, [v]))
        groups[name] = assigns
    return groups
