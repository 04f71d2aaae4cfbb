"""Portable solved fields: a cache entry exported as one .field.npz with the
producing spec's JSON beside it, and reinstated from one (ion_gym
io/field_io.py:185-930), in the reference's format, so bundles written here
open in the reference and the other way round.

Bundle members (np.savez_compressed):
    __bundle_version   int64 [1]
    __key              uint8, the entry key's ASCII
    arr__<name>        every <name>.npy of the entry, verbatim
    json__<name>       every <name>.json of the entry (meta, provenance),
                       its bytes as uint8
Beside it, <name>__<key8>.spec.json holds the producing spec (the latest
provenance record carrying spec_json), written first; both files are
published atomically.

GPU side: ``load_field_device`` reads a bundle's bases straight into a
CUDA float32 stack whose rows are 16-byte aligned (the layout the
superposition kernels read as float4), with the labels beside it, ready
for ``physics.field3d.compose_drive_channels``; ``store_device_bases``
writes device-resident unit bases as a cache entry.
"""
import json
import os
import re
import shutil
import tempfile
from pathlib import Path

import numpy as np

from ion_gym_gb300.io import fa_cache

FIELD_SUFFIX = ".field.npz"
V_BASIS = 1e4
_META = "_meta"
_SAFE = re.compile(r"[^A-Za-z0-9._-]+")


class FieldMismatch(ValueError):
    """A bundle that does not belong to the given geometry, or is not a
    field bundle in the current format."""


class FieldNotSolved(LookupError):
    """No solved entry in the cache to save."""


def _atomic_savez(path, **members):
    """npz written to a temporary name in the same folder, fsynced, then
    renamed into place (field_io.py:99-115)."""
    d = os.path.dirname(os.path.abspath(path)) or "."
    os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(prefix=".field_io.", suffix=".npz", dir=d)
    ok = False
    try:
        with os.fdopen(fd, "wb") as f:
            np.savez_compressed(f, **members)
            f.flush()
            os.fsync(f.fileno())
        os.replace(tmp, path)
        ok = True
    finally:
        if not ok and os.path.exists(tmp):
            os.remove(tmp)


def _atomic_write_text(path, text):
    d = os.path.dirname(os.path.abspath(path)) or "."
    os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(prefix=".field_io.", suffix=".tmp", dir=d)
    ok = False
    try:
        with os.fdopen(fd, "w", encoding="utf-8") as f:
            f.write(text)
            f.flush()
            os.fsync(f.fileno())
        os.replace(tmp, path)
        ok = True
    finally:
        if not ok and os.path.exists(tmp):
            os.remove(tmp)


def geometry_diff(a, b, prefix=""):
    """['path: A vs B', ...] between two geometry dicts
    (field_io.py:136-170): absent keys, list lengths and differing leaves,
    each named by its path."""
    out = []
    if isinstance(a, dict) and isinstance(b, dict):
        for k in sorted(set(a) | set(b)):
            if k not in a:
                out.append(f"{prefix}{k}: <absent> vs present")
            elif k not in b:
                out.append(f"{prefix}{k}: present vs <absent>")
            else:
                out.extend(geometry_diff(a[k], b[k], f"{prefix}{k}."))
    elif isinstance(a, list) and isinstance(b, list):
        if len(a) != len(b):
            out.append(f"{prefix.rstrip('.')}: length {len(a)} vs {len(b)}")
        else:
            for i, (x, y) in enumerate(zip(a, b)):
                out.extend(geometry_diff(x, y, f"{prefix}[{i}]."))
    elif a != b:
        out.append(f"{prefix.rstrip('.')}: {a!r} vs {b!r}")
    return out


def _root(root):
    return Path(root if root is not None else fa_cache.cache_root()).expanduser()


def entry_spec_json(key, root=None):
    """The latest provenance record's spec_json of an entry, None without a
    provenance file; an unreadable provenance file is refused
    (field_io.py:747-768)."""
    pp = _root(root) / key / "provenance.json"
    if not pp.exists():
        return None
    try:
        recs = json.loads(pp.read_text(encoding="utf-8"))
    except (OSError, ValueError) as e:
        raise ValueError(
            f"cache entry {key}: provenance record {pp} is unreadable "
            f"({type(e).__name__}: {e}) -- the entry's producing spec is "
            f"unknown; remove the entry (Cache tab) and re-solve") from e
    for r in reversed(recs if isinstance(recs, list) else []):
        if isinstance(r, dict) and r.get("spec_json"):
            return r["spec_json"]
    return None


def _spec_dict(spec):
    return spec.to_dict() if hasattr(spec, "to_dict") else spec


def resolve_cache_entry(spec, root=None):
    """The key of the one entry whose stored spec geometry equals this
    spec's (field_io.py:771-796)."""
    want = _spec_dict(spec)["geometry"]
    hits, legacy = [], 0
    for e in fa_cache.entries(root=root):
        sj = entry_spec_json(e["key"], root=root)
        if sj is None:
            legacy += 1
            continue
        if not geometry_diff(want, sj.get("geometry", {})):
            hits.append(e["key"])
    if len(hits) == 1:
        return hits[0]
    if not hits:
        raise FileNotFoundError(
            f"resolve_cache_entry: no cache entry matches the geometry of "
            f"{getattr(spec, 'name', '?')!r} ({legacy} legacy entries "
            f"without descriptors were skipped). Solve first (build_run); "
            f"legacy entries gain descriptors on their next solve.")
    raise ValueError(
        f"resolve_cache_entry: {len(hits)} entries share this geometry "
        f"({[h[:8] for h in hits]}) — export by key instead.")


def export_field_bundle(spec_or_key, out_dir, root=None):
    """Entry -> <name>__<key8>.field.npz (+ .spec.json); returns the two
    paths (the second None without a recorded spec).  Never solves
    (field_io.py:799-842)."""
    key = spec_or_key if isinstance(spec_or_key, str) else \
        resolve_cache_entry(spec_or_key, root=root)
    src = _root(root) / key
    if not src.is_dir():
        raise FileNotFoundError(f"export_field_bundle: cache entry {key} does not exist.")
    sj = entry_spec_json(key, root=root)
    name = ((sj or {}).get("name") or "field").replace(" ", "_")[:40]
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    stem = f"{name}__{key[:8]}"
    payload = {"__bundle_version": np.array([1]),
               "__key": np.frombuffer(key.encode(), np.uint8)}
    for f in sorted(src.iterdir()):
        if f.suffix == ".npy":
            payload[f"arr__{f.stem}"] = np.load(f)
        elif f.suffix == ".json":
            payload[f"json__{f.stem}"] = np.frombuffer(f.read_bytes(), np.uint8)
    npz = out / f"{stem}{FIELD_SUFFIX}"
    spec_path = None
    if sj is not None:
        spec_path = out / f"{stem}.spec.json"
        _atomic_write_text(spec_path, json.dumps(sj, indent=1))
    _atomic_savez(str(npz), **payload)
    return str(npz), (str(spec_path) if spec_path else None)


def import_field_bundle(path, spec=None, root=None):
    """Bundle -> cache entry under root, staged in a temporary folder with
    meta.json written last and published by one rename; a complete entry
    already there is kept, a partial one replaced.  With `spec`, refuses
    unless its geometry equals the bundle's recorded spec geometry
    (field_io.py:845-930).  Returns the key."""
    z = np.load(path, allow_pickle=False)
    if "__bundle_version" not in z:
        raise ValueError(
            f"import_field_bundle: {path} is not a field bundle (no "
            f"version tag) — array-level fields go through load_field.")
    key = bytes(z["__key"]).decode()
    if spec is not None:
        sj = None
        if "json__provenance" in z.files:
            recs = json.loads(bytes(z["json__provenance"]).decode())
            for r in reversed(recs if isinstance(recs, list) else []):
                if isinstance(r, dict) and r.get("spec_json"):
                    sj = r["spec_json"]
                    break
        if sj is None:
            raise ValueError(
                "import_field_bundle: a spec was given for validation but "
                "the bundle carries no producing-spec record (pre-"
                "descriptor entry) — import by trust is refused; pass "
                "spec=None only if you know the provenance.")
        diff = geometry_diff(_spec_dict(spec)["geometry"], sj.get("geometry", {}))
        if diff:
            raise ValueError(
                f"import_field_bundle: geometry mismatch — the bundle was "
                f"solved for different geometry. Differing fields: "
                f"{diff}. Refusing; load the spec JSON exported beside "
                f"the bundle, or re-solve.")
    if "json__meta" not in z.files:
        raise ValueError(
            f"import_field_bundle: {path} carries no meta.json -- the "
            f"entry's completeness marker; refusing a partial bundle")
    base = _root(root)
    dest = base / key
    if (dest / "meta.json").exists():
        return key
    base.mkdir(parents=True, exist_ok=True)
    tmp = Path(tempfile.mkdtemp(prefix=f".{key}.import.", dir=base))
    try:
        for k in z.files:
            if k.startswith("arr__"):
                np.save(tmp / f"{k[5:]}.npy", z[k])
        for k in z.files:
            if k.startswith("json__") and k != "json__meta":
                (tmp / f"{k[6:]}.json").write_bytes(bytes(z[k]))
        with open(tmp / "meta.json", "wb") as fh:
            fh.write(bytes(z["json__meta"]))
            fh.flush()
            os.fsync(fh.fileno())
        if dest.exists():
            shutil.rmtree(dest)
        os.replace(tmp, dest)
    finally:
        if tmp.exists():
            shutil.rmtree(tmp, ignore_errors=True)
    return key


def is_field_bundle(path):
    with np.load(path) as z:
        return "__bundle_version" in z.files


def read_field_meta(path):
    """{key, spec, spec_name} of a bundle from its small members
    (field_io.py:230-253)."""
    name = os.path.basename(path)
    with np.load(path) as z:
        if "__bundle_version" not in z.files:
            if _META in z.files:
                raise FieldMismatch(
                    f"{name} is in the older field format, which this "
                    f"version no longer reads. Solve the deck and save the "
                    f"field again.")
            raise FieldMismatch(f"{name} is not an ion_gym field file "
                                f"(members: {sorted(z.files)[:6]})")
        key = bytes(z["__key"]).decode()
        sj = None
        if "json__provenance" in z.files:
            recs = json.loads(bytes(z["json__provenance"]).decode())
            for r in reversed(recs if isinstance(recs, list) else []):
                if isinstance(r, dict) and r.get("spec_json"):
                    sj = r["spec_json"]
                    break
    return {"key": key, "spec": sj, "spec_name": (sj or {}).get("name")}


def read_field_arrays(path):
    """(bases {k: float64 per volt}, labels, meta) of a bundle
    (field_io.py:276-306): 3-D entries keep basis_<k> per volt, planar and
    r-z entries b<k> at V_BASIS."""
    meta = read_field_meta(path)
    bases, labels = {}, None
    with np.load(path) as z:
        for name in z.files:
            if not name.startswith("arr__"):
                continue
            arr = name[5:]
            if arr in ("ele", "labels"):
                labels = z[name]
            elif arr.startswith("basis_") and arr[6:].isdigit():
                bases[int(arr[6:])] = np.asarray(z[name], np.float64)
            elif arr.startswith("b") and arr[1:].isdigit():
                bases[int(arr[1:])] = z[name] / V_BASIS
    if not bases or labels is None:
        raise FieldMismatch(f"{os.path.basename(path)}: no bases or "
                            f"labels in the file")
    return dict(sorted(bases.items())), labels, meta


def save_field(key, directory, label=None, root=None):
    """Export a solved entry (by key) into `directory`; `label` goes to the
    folder's label registry (field_io.py:205-220)."""
    if fa_cache.load(key, root=root)[0] is None:
        raise FieldNotSolved(
            f"no solved field in the cache (entry {key[:8]}). Solve it "
            f"first, then save.")
    npz, deck = export_field_bundle(key, directory, root=root)
    if label:
        set_label(key, label, directory=directory)
    return npz, deck


def _registry_path(directory):
    return os.path.join(directory, "fields_registry.json")


def get_label(key, directory):
    try:
        with open(_registry_path(directory), encoding="utf-8") as f:
            return (json.load(f) or {}).get(key)
    except (OSError, ValueError):
        return None


def set_label(key, label, directory):
    path = _registry_path(directory)
    try:
        with open(path, encoding="utf-8") as f:
            reg = json.load(f) or {}
    except (OSError, ValueError):
        reg = {}
    if label:
        reg[key] = label
    else:
        reg.pop(key, None)
    _atomic_write_text(path, json.dumps(reg, indent=1, sort_keys=True))


# ------------------------------------------------------------------ device
def load_field_device(path, device="cuda"):
    """(stack, labels, keys, meta) of a 3-D bundle on the GPU: the unit
    bases as a float32 (n, nx, ny, nz) CUDA tensor with 16-byte-aligned rows
    (basis keys[r] in row r), the labels as a CUDA uint8 tensor."""
    from ion_gym_gb300.physics.field3d import padded
    import torch
    meta = read_field_meta(path)
    with np.load(path) as z:
        names = sorted((int(n[11:]), n) for n in z.files
                       if n.startswith("arr__basis_") and n[11:].isdigit())
        if not names or "arr__labels" not in z.files:
            raise FieldMismatch(f"{os.path.basename(path)}: not a 3-D field "
                                f"bundle (no basis_<k> / labels)")
        lab = z["arr__labels"]
        stack = padded(len(names), lab.shape, torch.float32, device)
        for r, (_, n) in enumerate(names):
            stack[r].copy_(torch.from_numpy(np.ascontiguousarray(z[n], np.float32)))
        labels = torch.from_numpy(np.ascontiguousarray(lab)).to(device)
    return stack, labels, [k for k, _ in names], meta


def store_device_bases(spec, stack, keys, labels, root=None, name=None,
                       label=None, spec_json=None):
    """Write device-resident unit bases (rows of `stack` for electrode
    indices `keys`) and labels as a cache entry in the 3-D layout
    (build_stl3d.py:919-924); with `name`, record provenance.  Returns the
    key."""
    arrays = {f"basis_{k}": stack[r].detach().cpu().numpy().astype(np.float32, copy=False)
              for r, k in enumerate(keys)}
    lab = labels.detach().cpu().numpy() if hasattr(labels, "detach") else np.asarray(labels)
    arrays["labels"] = np.ascontiguousarray(lab, np.uint8)
    key = fa_cache.store(spec, arrays, root=root)
    if name:
        fa_cache.annotate(key, name, label=label, root=root, spec_json=spec_json)
    return key
