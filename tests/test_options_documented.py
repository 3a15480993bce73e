"""Every context option the C ABI accepts (thc_ctx_set_option) is documented in the public
header, and every documented option is accepted (a source-level check, no GPU)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _read(*parts):
    with open(os.path.join(ROOT, *parts)) as f:
        return f.read()


def test_header_documents_every_option():
    accepted = set(re.findall(r'strcmp\(key, "([a-z0-9_]+)"\)',
                              _read("thcpp_gb300", "csrc", "capi.cu")))
    hdr = _read("include", "thc_gb300.h")
    block = hdr[hdr.index("Named numeric options"):hdr.index("int thc_ctx_set_option")]
    documented = set(re.findall(r'"([a-z0-9_]+)"', block))
    assert accepted, "no options found in capi.cu"
    assert accepted == documented, (sorted(accepted - documented), sorted(documented - accepted))
