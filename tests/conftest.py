import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
for p in (ROOT / "jax-sgmc_gb300", ROOT):
  if str(p) not in sys.path:
    sys.path.insert(0, str(p))


def pytest_configure(config):
  config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def _cuda_available() -> bool:
  try:
    import torch
    return torch.cuda.is_available()
  except Exception:  # pragma: no cover
    return False


def pytest_collection_modifyitems(config, items):
  if _cuda_available():
    return
  skip = pytest.mark.skip(reason="no CUDA device in this environment")
  for item in items:
    if "gpu" in item.keywords:
      item.add_marker(skip)


@pytest.fixture(scope="session")
def lib():
  """The CUDA library, built for sm_103a if needed."""
  from gbsgmc import _build, _lib
  _build.build()
  return _lib.load()
