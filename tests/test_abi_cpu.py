"""The C-ABI library loads and exports every symbol include/*.h declares."""
import re
from pathlib import Path

from cochlearmodel_gb300 import native

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b([A-Za-z_]\w*)\s*\(", text):
            name = m.group(1)
            # function declarations: identifier preceded by a return type
            pre = text[:m.start()].rstrip()
            if re.search(r"(\bvoid|\bint|\bint64_t|\bchar\s*\*|\bfloat\s*\*|\bint\s*\*|"
                         r"\bJNDFloat\s*\*|\bfloat|\bdouble)\s*\**$", pre):
                names.add(name)
    return names


def test_library_loads():
    lib = native.load()
    assert lib.cgb_abi_version() == 1


def test_every_declared_symbol_is_exported():
    lib = native.load()
    syms = declared_symbols()
    assert "cgb_bm_run_dev" in syms and "cgb_model_setup" in syms
    missing = [s for s in sorted(syms) if not hasattr(lib, s)]
    assert not missing, missing


def test_error_reporting():
    import pytest
    lib = native.load()
    with pytest.raises(native.CGBError, match="bad arguments"):
        native.check(lib.cgb_block_partition(0, 10, 0, 0, None, None, None), "partition")
