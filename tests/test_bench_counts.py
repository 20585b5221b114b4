"""The roofline counts in bench.py are keyed to the kernel code they were
measured on (DENSITY_NCU["sources"]): the key ignores comments, trailing blanks
and empty lines, and any code edit changes it, so that the bench line marks the
counts stale after a kernel change but not after a comment edit."""
import os
import shutil

import bench


def _copy_sources(root):
    for f in bench.KERNEL_SOURCES:
        dst = root / f
        dst.parent.mkdir(parents=True, exist_ok=True)
        shutil.copy(os.path.join(bench.ROOT, f), dst)


def test_key_ignores_comments_and_follows_code(tmp_path, monkeypatch):
    _copy_sources(tmp_path)
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    key = bench.kernel_sources_sha()
    src = tmp_path / bench.KERNEL_SOURCES[0]
    text = src.read_text(encoding="utf-8")
    commented = "// a new comment\n\n" + text.replace(";\n", ";  // note\n", 5) + "\n/* a block\n   comment */\n"
    src.write_text(commented, encoding="utf-8")
    assert bench.kernel_sources_sha() == key
    assert "constexpr int kThreads = 256;" in text
    src.write_text(text.replace("constexpr int kThreads = 256;", "constexpr int kThreads = 128;", 1),
                   encoding="utf-8")
    assert bench.kernel_sources_sha() != key
