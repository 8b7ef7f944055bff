"""fluid.cu as host C++ for the CTA emulation of tests/emu (test
infrastructure): kernel launches become emu_launch calls, dynamic shared
memory the emulated CTA's buffer, static shared arrays function statics
(the emulation runs one CTA at a time), the constant-memory thermodynamic
table a plain global."""
import re


def host_source(cu: str) -> str:
    def launch(m):
        return f"emu_launch({m.group(1)}, {m.group(2)}, {m.group(3)});"

    s = re.sub(r"(\w+)<<<(.+?)>>>\((.*?)\);", launch, cu, flags=re.S)
    s = re.sub(r"extern __shared__ double (\w+)\[\];", r"double* \1 = emu_sm;", s)
    s = re.sub(r"(?<!extern )__shared__ ", "static ", s)
    s = s.replace("__constant__ ThermoTable c_thermo;", "ThermoTable c_thermo;")
    s = s.replace("#include <cuda_runtime.h>", "")
    if "<<<" in s or "__shared__" in s or "__constant__" in s:
        raise ValueError("fluid.cu holds a construct the emulation does not translate")
    return s
