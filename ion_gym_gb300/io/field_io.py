"""Portable solved fields: a basis-cache entry packed into one .field.npz
with the producing spec's JSON beside it, and unpacked back into a cache
(ion_gym io/field_io.py:185-930), in the reference's bundle format, so
bundles written here open in the reference and the other way round.

Bundle members (np.savez_compressed):
    __bundle_version   int64 [1]
    __key              uint8, the entry key's ASCII
    arr__<name>        every <name>.npy of the entry, verbatim
    json__<name>       every <name>.json of the entry (meta, provenance),
                       its bytes as uint8
Beside it, <name>__<key8>.spec.json holds the producing spec (the newest
provenance record carrying spec_json).  Both files are published through
io.publish (temporary name, sync, rename).

The file <-> member mapping is the table CODECS: packing walks the entry's
files and looks each suffix up, unpacking walks the members and looks each
prefix up; meta.json, the entry's completeness marker, is always written
last.

GPU side: ``load_field_device`` reads a bundle's bases straight into a
CUDA float32 stack whose rows are 16-byte aligned (the layout the
superposition kernels read as float4), with the labels beside it, ready
for ``physics.field3d.compose_drive_channels``; ``store_device_bases``
writes device-resident unit bases as a cache entry.
"""
import json
import os
from pathlib import Path
from typing import Callable, NamedTuple

import numpy as np

from ion_gym_gb300.io import fa_cache
from ion_gym_gb300.io.publish import staged, write_json, write_npz, write_text

FIELD_SUFFIX = ".field.npz"
BUNDLE_VERSION = 1
V_BASIS = 1e4                 # the planar / r-z bases are cached at this
_HEADER = ("__bundle_version", "__key")
_OLD_FORMAT_MEMBER = "_meta"  # the single member of the older field files


class FieldMismatch(ValueError):
    """A file that is not a field bundle in the current format, or one that
    does not belong to the given geometry."""


class FieldNotSolved(LookupError):
    """No solved entry in the cache to save."""


# ------------------------------------------------------------------ codec
class Codec(NamedTuple):
    prefix: str                                 # bundle member prefix
    suffix: str                                 # entry file suffix
    pack: Callable[[Path], np.ndarray]          # file -> member
    unpack: Callable[[np.ndarray, Path], None]  # member -> file


def _bytes_member(path):
    return np.frombuffer(path.read_bytes(), np.uint8)


def _member_bytes(arr):
    return np.ascontiguousarray(arr, np.uint8).tobytes()


CODECS = (
    Codec("arr__", ".npy", lambda p: np.load(p, allow_pickle=False),
          lambda a, p: np.save(p, a)),
    Codec("json__", ".json", _bytes_member,
          lambda a, p: p.write_bytes(_member_bytes(a))),
)


def _codec_of_member(member):
    for c in CODECS:
        if member.startswith(c.prefix):
            return c
    return None


def _codec_of_file(path):
    for c in CODECS:
        if path.suffix == c.suffix:
            return c
    return None


def pack_entry(entry_dir, key):
    """{member: array} of a cache entry folder: the header and one member
    per .npy / .json file, in file-name order."""
    members = {"__bundle_version": np.array([BUNDLE_VERSION]),
               "__key": np.frombuffer(key.encode("ascii"), np.uint8)}
    for f in sorted(Path(entry_dir).iterdir()):
        c = _codec_of_file(f)
        if c is not None and f.is_file():
            members[c.prefix + f.stem] = c.pack(f)
    return members


def unpack_members(z, dest_dir):
    """Write every codec member of bundle `z` into `dest_dir`, meta.json
    (the completeness marker) last."""
    dest_dir = Path(dest_dir)
    names = [m for m in z.files if _codec_of_member(m) is not None]
    names.sort(key=lambda m: m == "json__meta")
    for m in names:
        c = _codec_of_member(m)
        c.unpack(z[m], dest_dir / (m[len(c.prefix):] + c.suffix))


def _json_member(z, member):
    return json.loads(_member_bytes(z[member]).decode("utf-8"))


def _bundle_spec(z):
    """The producing spec recorded in a bundle's provenance member."""
    if "json__provenance" not in z.files:
        return None
    recs = _json_member(z, "json__provenance")
    if not isinstance(recs, list):
        return None
    return fa_cache.latest_spec_json([r for r in recs if isinstance(r, dict)])


# -------------------------------------------------------------- geometry
def _divergences(a, b):
    """(path, detail) of every place two JSON-like trees differ, depth first
    with dict keys in sorted order (an explicit stack, so deep trees do not
    recurse)."""
    stack = [((), a, b)]
    while stack:
        path, x, y = stack.pop()
        if path is None:              # a note queued in order
            yield x, y
            continue
        if isinstance(x, dict) and isinstance(y, dict):
            todo = []
            for k in sorted(set(x) | set(y)):
                p = path + (str(k),)
                if k not in x:
                    todo.append((None, p, "<absent> vs present"))
                elif k not in y:
                    todo.append((None, p, "present vs <absent>"))
                else:
                    todo.append((p, x[k], y[k]))
            stack.extend(reversed(todo))
        elif isinstance(x, list) and isinstance(y, list):
            if len(x) != len(y):
                yield path, f"length {len(x)} vs {len(y)}"
            else:
                stack.extend(reversed([(path + (f"[{i}]",), u, v)
                                       for i, (u, v) in enumerate(zip(x, y))]))
        elif x != y:
            yield path, f"{x!r} vs {y!r}"


def geometry_diff(a, b):
    """['path: A vs B', ...]: where two geometry dicts differ -- a key on
    one side only, a list length, or a differing leaf -- each named by its
    path ('electrodes.[1].v'), in the order of the reference's report
    (field_io.py:136-170)."""
    return [f"{'.'.join(p)}: {d}" for p, d in _divergences(a, b)]


# ------------------------------------------------------------------ cache
def _root(root):
    return Path(root if root is not None else fa_cache.cache_root()).expanduser()


def entry_spec_json(key, root=None):
    """The producing spec recorded in an entry's provenance (None when it
    has no provenance file); an unreadable provenance file is refused,
    since the entry's origin is then unknown (field_io.py:747-768)."""
    entry = _root(root) / key
    recs, why = fa_cache._records(str(entry))
    if why is not None:
        raise ValueError(
            f"cache entry {key}: its provenance record cannot be read "
            f"({why}), so the spec that produced it is unknown; delete the "
            f"entry and solve again")
    return fa_cache.latest_spec_json(recs)


def _spec_dict(spec):
    return spec.to_dict() if hasattr(spec, "to_dict") else spec


def resolve_cache_entry(spec, root=None):
    """The key of the single entry whose recorded spec has this spec's
    geometry (field_io.py:771-796).  Entries without a recorded spec are
    skipped; no match raises FileNotFoundError, several raise ValueError."""
    want = _spec_dict(spec)["geometry"]
    hits, unrecorded = [], 0
    for row in fa_cache.entries(root=root):
        sj = entry_spec_json(row["key"], root=root)
        if sj is None:
            unrecorded += 1
        elif not geometry_diff(want, sj.get("geometry", {})):
            hits.append(row["key"])
    if len(hits) == 1:
        return hits[0]
    name = getattr(spec, "name", None) or _spec_dict(spec).get("name", "?")
    if not hits:
        raise FileNotFoundError(
            f"resolve_cache_entry: no cache entry was solved for the "
            f"geometry of {name!r} ({unrecorded} entries without a recorded "
            f"spec were not compared); solve it first")
    raise ValueError(
        f"resolve_cache_entry: {len(hits)} entries hold this geometry "
        f"({', '.join(h[:8] for h in hits)}); export one by its key")


# --------------------------------------------------------------- bundles
def export_field_bundle(spec_or_key, out_dir, root=None):
    """Pack an entry (by key, or the one matching a spec's geometry) into
    <name>__<key8>.field.npz in out_dir, with <name>__<key8>.spec.json
    beside it when a producing spec is recorded.  Never solves.  Returns
    (bundle path, spec path or None) (field_io.py:799-842)."""
    key = (spec_or_key if isinstance(spec_or_key, str)
           else resolve_cache_entry(spec_or_key, root=root))
    entry = _root(root) / key
    if not entry.is_dir():
        raise FileNotFoundError(f"export_field_bundle: no cache entry {key}")
    sj = entry_spec_json(key, root=root)
    stem = ((sj or {}).get("name") or "field").replace(" ", "_")[:40]
    stem = f"{stem}__{key[:8]}"
    out = Path(out_dir)
    spec_path = None
    if sj is not None:
        spec_path = out / f"{stem}.spec.json"
        write_json(spec_path, sj)
    bundle = out / f"{stem}{FIELD_SUFFIX}"
    write_npz(bundle, pack_entry(entry, key))
    return str(bundle), (str(spec_path) if spec_path else None)


def _check_bundle(z, path):
    if "__bundle_version" in z.files:
        return
    name = os.path.basename(str(path))
    if _OLD_FORMAT_MEMBER in z.files:
        raise FieldMismatch(
            f"{name} uses the older field format (one {_OLD_FORMAT_MEMBER} "
            f"member), which this version does not read; solve the deck and "
            f"save the field again")
    raise FieldMismatch(
        f"{name} is not an ion_gym field file: it has no bundle header "
        f"(members: {sorted(z.files)[:6]})")


def import_field_bundle(path, spec=None, root=None):
    """Unpack a bundle into the cache under root and return its key
    (field_io.py:845-930).  The entry is staged in a temporary folder and
    published by one rename; a complete entry already there is kept, a
    partial one replaced.  With `spec`, the bundle's recorded producing
    spec must have the same geometry, else ValueError (a bundle without a
    recorded spec is refused too)."""
    with np.load(path, allow_pickle=False) as z:
        if "__bundle_version" not in z.files:
            raise ValueError(
                f"import_field_bundle: {path} has no bundle header, so it is "
                f"not a field bundle")
        key = _member_bytes(z["__key"]).decode("ascii")
        if spec is not None:
            sj = _bundle_spec(z)
            if sj is None:
                raise ValueError(
                    "import_field_bundle: a spec was given to validate "
                    "against, but the bundle records no producing spec; "
                    "import it without a spec only if its origin is known")
            diff = geometry_diff(_spec_dict(spec)["geometry"],
                                 sj.get("geometry", {}))
            if diff:
                # the wording of this refusal is the reference's
                raise ValueError(
                    f"import_field_bundle: geometry mismatch — the bundle was "
                    f"solved for different geometry. Differing fields: "
                    f"{diff}. Refusing; load the spec JSON exported beside "
                    f"the bundle, or re-solve.")
        if "json__meta" not in z.files:
            raise ValueError(
                f"import_field_bundle: {path} has no meta.json member, the "
                f"entry's completeness marker; a partial bundle is refused")
        dest = _root(root) / key
        if not fa_cache._complete(str(dest)):
            with staged(dest, folder=True, keep_if=fa_cache._complete) as tmp:
                unpack_members(z, tmp)
    return key


def is_field_bundle(path):
    with np.load(path, allow_pickle=False) as z:
        return "__bundle_version" in z.files


def read_field_meta(path):
    """{key, spec, spec_name} of a bundle, from its small members
    (field_io.py:230-253); FieldMismatch for an older-format field file or
    any other npz."""
    with np.load(path, allow_pickle=False) as z:
        _check_bundle(z, path)
        key = _member_bytes(z["__key"]).decode("ascii")
        sj = _bundle_spec(z)
    return {"key": key, "spec": sj, "spec_name": (sj or {}).get("name")}


def _array_role(arr):
    """('labels', None), ('per_volt', k), ('at_v_basis', k) or (None, None)
    for a bundle array name: 3-D entries keep basis_<k> per volt, planar
    and r-z entries b<k> as solved at V_BASIS; their labels are 'labels'
    and 'ele'."""
    if arr in ("labels", "ele"):
        return "labels", None
    for head, role in (("basis_", "per_volt"), ("b", "at_v_basis")):
        tail = arr[len(head):]
        if arr.startswith(head) and tail.isdigit():
            return role, int(tail)
    return None, None


def read_field_arrays(path):
    """(bases {k: float64 potential per volt}, labels, meta) of a bundle
    (field_io.py:276-306)."""
    meta = read_field_meta(path)
    bases, labels = {}, None
    with np.load(path, allow_pickle=False) as z:
        for m in z.files:
            if not m.startswith("arr__"):
                continue
            role, k = _array_role(m[5:])
            if role == "labels":
                labels = z[m]
            elif role == "per_volt":
                bases[k] = np.asarray(z[m], np.float64)
            elif role == "at_v_basis":
                bases[k] = z[m] / V_BASIS
    if not bases or labels is None:
        raise FieldMismatch(f"{os.path.basename(path)}: the bundle holds no "
                            f"bases or no labels")
    return dict(sorted(bases.items())), labels, meta


def save_field(key, directory, label=None, root=None):
    """Export a solved entry (by key) into `directory`, never solving;
    `label` goes to that folder's label registry (field_io.py:205-220)."""
    if fa_cache.load(key, root=root)[0] is None:
        raise FieldNotSolved(
            f"cache entry {key[:8]} holds no solved field to save; solve the "
            f"deck first")
    paths = export_field_bundle(key, directory, root=root)
    if label:
        set_label(key, label, directory=directory)
    return paths


# ------------------------------------------------------- label registry
def _registry(directory):
    path = os.path.join(directory, "fields_registry.json")
    reg, _ = fa_cache._read_json(path)
    return path, (reg if isinstance(reg, dict) else {})


def get_label(key, directory):
    return _registry(directory)[1].get(key)


def set_label(key, label, directory):
    """Set (or, with an empty label, clear) the label of `key` in the
    folder's fields_registry.json."""
    path, reg = _registry(directory)
    reg.pop(key, None)
    if label:
        reg[key] = label
    write_text(path, json.dumps(reg, indent=1, sort_keys=True))


# ------------------------------------------------------------------ device
def load_field_device(path, device="cuda"):
    """(stack, labels, keys, meta) of a 3-D bundle on the GPU: the unit
    bases as a float32 (n, nx, ny, nz) CUDA tensor with 16-byte-aligned rows
    (basis keys[r] in row r), the labels as a CUDA uint8 tensor."""
    from ion_gym_gb300.physics.field3d import padded
    import torch
    meta = read_field_meta(path)
    with np.load(path, allow_pickle=False) as z:
        rows = sorted((k, m) for m in z.files if m.startswith("arr__")
                      for role, k in [_array_role(m[5:])] if role == "per_volt")
        if not rows or "arr__labels" not in z.files:
            raise FieldMismatch(f"{os.path.basename(path)}: not a 3-D field "
                                f"bundle (no basis_<k> / labels)")
        lab = z["arr__labels"]
        stack = padded(len(rows), lab.shape, torch.float32, device)
        for r, (_, m) in enumerate(rows):
            stack[r].copy_(torch.from_numpy(np.ascontiguousarray(z[m], np.float32)))
        labels = torch.from_numpy(np.ascontiguousarray(lab)).to(device)
    return stack, labels, [k for k, _ in rows], meta


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
