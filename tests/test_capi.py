"""The C-ABI library: builds, loads, exports every declared symbol, and its
settings struct is byte-identical to pRRTC_settings (CPU, no GPU calls)."""
import ctypes as C
import re

from conftest import ROOT


def declared_functions():
    text = (ROOT / "include/prrtc/prrtc.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(prrtc_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    import prrtc_gb300.build as b
    lib = C.CDLL(str(b.build()))
    names = declared_functions()
    assert len(names) >= 17
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []


def test_settings_layout_matches_reference():
    from prrtc_gb300.api import Settings
    # pRRTC_settings.hh:3-16: int,int,int,int,float,int,float,bool,float,float,float
    offs = {n: getattr(Settings, n).offset for n, _ in Settings._fields_}
    assert offs == {"max_samples": 0, "max_iters": 4, "num_new_configs": 8, "granularity": 12, "range": 16,
                    "balance": 20, "tree_ratio": 24, "dynamic_domain": 28, "dd_alpha": 32, "dd_radius": 36,
                    "dd_min_radius": 40}
    assert C.sizeof(Settings) == 44
    s = Settings()
    assert (s.max_samples, s.num_new_configs, s.granularity, s.balance, s.dynamic_domain) == (1000000, 600, 64, 1, True)


def test_robot_tables():
    from prrtc_gb300 import api
    assert [api.dof(r) for r in ("sphere", "panda", "fetch", "baxter")] == [3, 7, 8, 14]
    assert [api.num_spheres(r) for r in ("sphere", "panda", "fetch", "baxter")] == [1, 69, 125, 100]


def test_struct_layouts_match_the_header(tmp_path):
    """ctypes mirrors of the ABI structs have the header's size and offsets."""
    import subprocess
    from prrtc_gb300 import api
    structs = {"prrtc_settings": api.Settings, "prrtc_result": api._Result, "prrtc_env_desc": api.EnvDesc,
               "prrtc_query": api._Query, "prrtc_batch_settings": api.BatchSettings,
               "prrtc_batch_stats": api._BatchStats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "prrtc/prrtc.h"', 'int main(void) {']
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    got = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n") if l)
    for cname, py in structs.items():
        assert int(got[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got[f"{cname}.{f}"]) == getattr(py, f).offset, f"{cname}.{f}"
