import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def native():
    """Builds the native libraries once per session."""
    from firepony_gb300 import build
    build.build_all()
    return build


def make_dataset(preset_name, num_reads, batch_reads, total_reference_bp=None, **kw):
    from firepony_gb300 import synth
    p = synth.PRESETS[preset_name].scaled(num_reads=num_reads, batch_reads=batch_reads,
                                          total_reference_bp=total_reference_bp, **kw)
    ref = synth.Reference(p)
    return p, ref, list(ref.batches())
