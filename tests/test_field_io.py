"""The portable field bundle (ion_gym io/field_io.py) against the
reference: tests/golden/bundle.npz holds a small 3-D entry written by the
reference's cache, the bundle its export made, what its reader returned and
what its import reinstated.  The same entry written here must export to the
same members and spec JSON, and the reference's bundle must import here to
the same files."""
import json
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, same_bits
from ion_gym_gb300.io import fa_cache, field_io

sys.path.insert(0, GOLDEN)
import make_golden as MG  # noqa: E402


@pytest.fixture(scope="module")
def gz():
    return np.load(os.path.join(GOLDEN, "bundle.npz"), allow_pickle=False)


def _prov(raw):
    recs = json.loads(bytes(raw).decode())
    for r in recs:
        r.pop("when", None)
    return recs


def _entry(tmp_path):
    spec, arrays, spec_json = MG.bundle_spec()
    root = str(tmp_path / "cache")
    key = fa_cache.store(spec, arrays, root=root)
    fa_cache.annotate(key, "ring deck", label="first", root=root,
                      spec_json=spec_json)
    return key, root


def test_export_matches_reference(tmp_path, gz):
    key, root = _entry(tmp_path)
    assert key == str(gz["bundle/0/key"])
    npz, deck = field_io.export_field_bundle(key, str(tmp_path / "out"), root=root)
    assert os.path.basename(npz) == str(gz["bundle/0/npz_name"])
    assert os.path.basename(deck) == str(gz["bundle/0/deck_name"])
    assert open(deck, encoding="utf-8").read() == str(gz["bundle/0/deck_text"])
    with np.load(npz) as z:
        assert sorted(z.files) == list(gz["bundle/0/members"])
        for m in z.files:
            want = gz[f"member/{m}/value"]
            if m == "json__provenance":
                assert _prov(z[m]) == _prov(want)
            else:
                assert z[m].dtype == want.dtype and same_bits(z[m], want), m


def _reference_bundle(gz, path):
    members = {m: gz[f"member/{m}/value"] for m in gz["bundle/0/members"]}
    np.savez_compressed(path, **members)
    return path


def test_reference_bundle_reads_and_imports(tmp_path, gz):
    npz = _reference_bundle(gz, str(tmp_path / "ref.field.npz"))
    assert field_io.is_field_bundle(npz)
    bases, labels, meta = field_io.read_field_arrays(npz)
    assert sorted(bases) == list(gz["bundle/0/read_keys"])
    for k, b in bases.items():
        assert b.dtype == np.float64 and same_bits(b, gz[f"read/{k}/basis"])
    assert same_bits(labels, gz["bundle/0/read_labels"])
    assert json.dumps(meta, sort_keys=True) == str(gz["bundle/0/meta_json"])
    root2 = str(tmp_path / "cache2")
    key = field_io.import_field_bundle(npz, root=root2)
    assert key == str(gz["bundle/0/import_key"])
    assert sorted(os.listdir(os.path.join(root2, key))) == list(gz["bundle/0/import_files"])
    with open(os.path.join(root2, key, "meta.json"), "rb") as f:
        assert f.read() == gz["bundle/0/import_meta_bytes"].tobytes()
    arrs, _ = fa_cache.load(key, root=root2)
    assert arrs is not None and same_bits(arrs["basis_1"], gz["member/arr__basis_1/value"])
    # importing again keeps the complete entry
    assert field_io.import_field_bundle(npz, root=root2) == key


def test_import_refuses_other_geometry(tmp_path, gz):
    npz = _reference_bundle(gz, str(tmp_path / "ref.field.npz"))
    _, _, spec_json = MG.bundle_spec()
    bad = dict(spec_json, geometry=dict(spec_json["geometry"], mm_per_gu=0.5))

    class S:
        def to_dict(self):
            return bad
    with pytest.raises(ValueError) as e:
        field_io.import_field_bundle(npz, spec=S(), root=str(tmp_path / "c3"))
    assert str(e.value) == str(gz["bundle_err/geometry/message"])


def test_refusals_and_labels(tmp_path):
    other = str(tmp_path / "x.npz")
    np.savez_compressed(other, a=np.zeros(3))
    with pytest.raises(field_io.FieldMismatch, match="not an ion_gym field file"):
        field_io.read_field_meta(other)
    np.savez_compressed(other, _meta=np.zeros(3, np.uint8))
    with pytest.raises(field_io.FieldMismatch, match="older field format"):
        field_io.read_field_meta(other)
    with pytest.raises(field_io.FieldNotSolved):
        field_io.save_field("0123456789abcdef", str(tmp_path / "o"),
                            root=str(tmp_path / "empty"))
    key, root = _entry(tmp_path)
    npz, _ = field_io.save_field(key, str(tmp_path / "o"), label="mine", root=root)
    assert field_io.get_label(key, str(tmp_path / "o")) == "mine"
    assert field_io.read_field_meta(npz)["spec_name"] == "ring deck"
    assert field_io.resolve_cache_entry({"geometry": MG.bundle_spec()[2]["geometry"]},
                                        root=root) == key


def test_geometry_diff_paths_and_order():
    a = {"mm_per_gu": 0.25, "electrodes": [{"name": "e1", "v": 1.0},
                                           {"name": "e2", "v": 2.0}],
         "grid": {"nx": 10, "ny": 12}, "only_a": 1}
    b = {"mm_per_gu": 0.25, "electrodes": [{"name": "e1", "v": 1.5},
                                           {"name": "e2", "v": 2.0, "w": 3}],
         "grid": {"nx": 10, "ny": [12]}, "only_b": 2}
    assert field_io.geometry_diff(a, b) == [
        "electrodes.[0].v: 1.0 vs 1.5",
        "electrodes.[1].w: <absent> vs present",
        "grid.ny: 12 vs [12]",
        "only_a: present vs <absent>",
        "only_b: <absent> vs present"]
    assert field_io.geometry_diff({"e": [1, 2]}, {"e": [1]}) == ["e: length 2 vs 1"]
    assert field_io.geometry_diff(a, a) == []


def test_inventory_and_provenance(tmp_path):
    key, root = _entry(tmp_path)
    fa_cache.annotate(key, "ring deck", label="first", root=root)    # refresh
    fa_cache.annotate(key, "other deck", label=None, root=root)
    fa_cache.annotate(key, "   ", root=root)                          # ignored
    recs = json.load(open(os.path.join(root, key, "provenance.json")))
    assert [(r["name"], r["label"]) for r in recs] == [("ring deck", "first"),
                                                       ("other deck", None)]
    assert "spec_json" in recs[0] and "spec_json" not in recs[1]
    (row,) = fa_cache.entries(root=root)
    assert row["key"] == key and row["arrays"] == 3 and row["problems"] == []
    assert row["produced_by"] == ["ring deck", "other deck"]
    assert row["descriptor"] == "first" and row["has_spec_json"]
    assert row["spec_name"] == "ring deck" and row["bytes"] > 0
    # an unreadable sidecar is reported by the inventory and started afresh
    # by the next annotation
    with open(os.path.join(root, key, "provenance.json"), "w") as f:
        f.write("{not json")
    (row,) = fa_cache.entries(root=root)
    assert row["produced_by"] == [] and "unreadable" in row["problems"][0]
    fa_cache.annotate(key, "again", root=root)
    assert [r["name"] for r in json.load(
        open(os.path.join(root, key, "provenance.json")))] == ["again"]
    assert fa_cache.entries(root=str(tmp_path / "none")) == []
