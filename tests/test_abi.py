"""The C ABI: the libraries load and export every symbol the headers declare."""
from __future__ import annotations

import re
import subprocess

from conftest import ROOT

HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared(header) -> set[str]:
    text = header.read_text()
    return set(re.findall(r"AXIOM_API\s+[\w\s\*]+?\b(\w+)\s*\(", text))


def exported(path) -> set[str]:
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True,
                         check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_headers_declare_entry_points():
    names = set().union(*(declared(h) for h in HEADERS))
    assert "axiom_world_step" in names and "axiom_world_create" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(lib):
    names = set().union(*(declared(h) for h in HEADERS))
    missing = names - exported(lib._name)
    assert not missing, f"declared but not exported: {sorted(missing)}"


def test_oracle_exports_the_world_abi(oracle):
    names = {n for n in declared(ROOT / "include" / "axiom_c.h") if n.startswith("axiom_world")}
    missing = names - exported(oracle._name)
    assert not missing, f"oracle lacks: {sorted(missing)}"


def test_config_defaults_match_reference(lib, oracle):
    """gui::PhysicsWorldConfig defaults (physics_panel.hpp:34-43) on both sides."""
    import axiom_gb300 as ax

    for l in (lib, oracle):
        c = ax.default_config(l)
        assert list(c.gravity) == [0.0, -9.8100004196167, 0.0] or abs(c.gravity[1] + 9.81) < 1e-6
        assert abs(c.time_step - 1.0 / 60.0) < 1e-9
        assert c.velocity_iterations == 8 and c.position_iterations == 3
        assert c.warm_start == ax.WARM_PREVIOUS


def test_version_strings(lib, oracle):
    assert b"sm_103a" in lib.axiom_version()
    assert b"oracle" in oracle.axiom_version()
