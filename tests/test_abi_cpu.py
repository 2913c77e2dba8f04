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
    assert lib.cgb_abi_version() == 4


# C++ templates of the reference API (include/cochlea_common.h:186-191) with the
# explicit instantiations the reference provides (src/cochlea.cu:747-760),
# exported under their Itanium-ABI names.
TEMPLATE_INSTANCES = {
    "GeneralKernel_Copy_Results_Template": [
        "_Z35GeneralKernel_Copy_Results_TemplateIfEvPT_S1_m",
        "_Z35GeneralKernel_Copy_Results_TemplateIdEvPT_S1_m",
        "_Z35GeneralKernel_Copy_Results_TemplateIiEvPT_S1_m",
        "_Z35GeneralKernel_Copy_Results_TemplateIfEvPT_S1_mm",
        "_Z35GeneralKernel_Copy_Results_TemplateIdEvPT_S1_mm",
        "_Z35GeneralKernel_Copy_Results_TemplateIiEvPT_S1_mm"],
    "ReverseKernel_Copy_Results_Template": [
        "_Z35ReverseKernel_Copy_Results_TemplateIfEvPT_S1_mmi",
        "_Z35ReverseKernel_Copy_Results_TemplateIdEvPT_S1_mmi"],
    "updateCUDALambdaArray": [
        "_Z21updateCUDALambdaArrayIfEvPT_S1_miiiiR3Log",
        "_Z21updateCUDALambdaArrayIdEvPT_S1_miiiiR3Log"],
}


def test_every_declared_symbol_is_exported():
    lib = native.load()
    syms = declared_symbols()
    assert "cgb_bm_run_dev" in syms and "cgb_model_setup" in syms
    assert "BMOHCNewKernel" in syms and "CudaCalculateJND" in syms
    missing = []
    for s in sorted(syms):
        names = TEMPLATE_INSTANCES.get(s, [s])
        missing += [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_error_reporting():
    import pytest
    lib = native.load()
    with pytest.raises(native.CGBError, match="bad arguments"):
        native.check(lib.cgb_block_partition(0, 10, 0, 0, None, None, None), "partition")
