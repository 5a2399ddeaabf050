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
