"""pizza's input.nml read into a Config and the run controls.

The groups and names are those of read_namelists (src/namelists.f90:162-189:
&grid, &control, &phys_param, &B.C., &start_field, &output_control); their
defaults are Config's (src/namelists.f90:530-672).  Names are matched without
regard to case, as Fortran does.  Names this library has no use for are
returned in ``ignored`` rather than rejected, so an existing input.nml reads
as it is; settings the step does not support are rejected by pz_create.
"""
import dataclasses
import re

from . import Config

# Config fields by their lower-case namelist names
_FIELDS = {f.name.lower(): f.name for f in dataclasses.fields(Config)}
# run controls (step_time.f90, outputs.f90, init_fields.f90)
_CONTROLS = {"n_time_steps", "n_log_step", "n_logs", "tag", "init_t", "amp_t", "init_xi", "amp_xi",
             "l_start_file", "start_file", "n_frame_step", "n_frames", "n_spec_step", "n_specs",
             "n_checkpoint_step", "n_checkpoints", "runhours", "runmin", "runsec", "tend"}

_LOGICALS = {".true.": True, ".false.": False, "t": True, "f": False, ".t.": True, ".f.": False}


def _value(tok: str):
    t = tok.strip()
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        return t[1:-1]
    low = t.lower()
    if low in _LOGICALS:
        return _LOGICALS[low]
    num = low.replace("d", "e")
    try:
        if re.fullmatch(r"[+-]?\d+", num):
            return int(num)
        return float(num)
    except ValueError:
        return t


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


def _split_items(body: str):
    """Split 'a = 1, b = 'x, y', c=.true.' at the commas and newlines outside quotes."""
    items, cur, quote = [], [], None
    for ch in body:
        if quote:
            if ch == quote:
                quote = None
            cur.append(ch)
        elif ch in "'\"":
            quote = ch
            cur.append(ch)
        elif ch in ",\n":
            items.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    items.append("".join(cur))
    # a value may be a list over several items: glue items without '=' to the previous one
    merged = []
    for it in items:
        if not it.strip():
            continue
        if "=" in it or not merged:
            merged.append(it)
        else:
            merged[-1] += "," + it
    return merged


def parse(text: str) -> dict:
    """{group (lower case): {name (lower case): value}} of a namelist file."""
    text = "\n".join(_strip_comment(ln) for ln in text.splitlines())
    groups = {}
    for m in re.finditer(r"&\s*([A-Za-z_][\w.]*)(.*?)(?:^\s*/|/\s*$|\$end)", text, re.S | re.M):
        name, body = m.group(1).lower(), m.group(2)
        vals = groups.setdefault(name, {})
        for item in _split_items(body):
            if "=" not in item:
                continue
            key, val = item.split("=", 1)
            parts = val.split(",") if "," in val and val.strip()[:1] not in ("'", '"') else [val]
            v = [_value(p) for p in parts]
            vals[key.strip().lower()] = v[0] if len(v) == 1 else v
    return groups


def read(path: str):
    """(Config, controls, ignored) of an input.nml file: the Config of the
    instance, the run controls (n_time_steps, n_log_step, tag, init_t, amp_t,
    start_file, ...) and the names this library does not use."""
    with open(path) as f:
        groups = parse(f.read())
    cfg, ctl, ignored = {}, {}, {}
    for g, vals in groups.items():
        for k, v in vals.items():
            if k in _FIELDS:
                cfg[_FIELDS[k]] = v
            elif k in _CONTROLS:
                ctl[k] = v
            else:
                ignored[f"{g}.{k}"] = v
    return Config(**cfg), ctl, ignored
