"""Host side of the per-phase timers (no GPU): the sweep driver brackets a phase only
while the current context's timers run, closes it when the phase raises, and the
phase names follow the C ABI's NSG_PHASE_* order."""
import re
from pathlib import Path

import pytest

from networksolvers_gb300 import _native, sweep

ROOT = Path(__file__).resolve().parent.parent


class _FakeCtx:
    def __init__(self, timing):
        self.timing = timing
        self.calls = []

    def phase(self, name, begin):
        self.calls.append((name, bool(begin)))


def test_phase_brackets_only_while_timing(monkeypatch):
    on, off = _FakeCtx(True), _FakeCtx(False)
    monkeypatch.setattr(_native, "current_context", lambda: on)
    with sweep._phase("krylov"):
        pass
    assert on.calls == [("krylov", True), ("krylov", False)]
    monkeypatch.setattr(_native, "current_context", lambda: off)
    with sweep._phase("krylov"):
        pass
    assert off.calls == []
    monkeypatch.setattr(_native, "current_context", lambda: None)
    with sweep._phase("extract"):
        pass


def test_phase_closes_on_error(monkeypatch):
    on = _FakeCtx(True)
    monkeypatch.setattr(_native, "current_context", lambda: on)
    with pytest.raises(ValueError):
        with sweep._phase("factorize"):
            raise ValueError("inserter failed")
    assert on.calls == [("factorize", True), ("factorize", False)]


def test_phase_names_follow_the_abi():
    hdr = (ROOT / "include" / "nsg.h").read_text()
    codes = {m.group(1).lower(): int(m.group(2)) for m in re.finditer(r"#define NSG_PHASE_(\w+) (\d+)", hdr)}
    ncount = codes.pop("ncount")
    assert ncount == len(_native.PHASES)
    assert [n for n, _ in sorted(codes.items(), key=lambda kv: kv[1])] == _native.PHASES
