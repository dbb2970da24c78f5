"""The library build is keyed by a hash of its sources, not by file times."""
import os

import pytest

from pyiid_gb300 import build as B


def test_stamp_matches_after_build():
    B.build()
    assert B.is_current()
    with open(B.stamp_path()) as f:
        assert f.read().strip() == B.source_hash()


def test_edited_source_invalidates_the_stamp(tmp_path, monkeypatch):
    B.build()
    extra = tmp_path / 'extra.cuh'
    extra.write_text('// one more header\n')
    srcs = B._sources() + [str(extra)]
    monkeypatch.setattr(B, '_sources', lambda: srcs)
    assert not B.is_current()
    # a newer modification time alone does not make the old library current
    extra.write_text('// edited\n')
    os.utime(B.lib_path(), None)
    assert not B.is_current()


def test_missing_stamp_is_not_current(monkeypatch, tmp_path):
    monkeypatch.setattr(B, 'stamp_path', lambda: str(tmp_path / 'none.sha256'))
    assert not B.is_current()
