"""Reference data access (mirrors jax_sgmc.data)."""

from .core import (CacheState, DataLoader, DeviceDataLoader, DeviceDataset,
                   FullDataMap, HostDataLoader, IndexedBatch,
                   MiniBatchInformation, RandomBatchFn, ShuffledFeed,
                   full_data_mapper,
                   full_reference_data, random_data_state,
                   random_reference_data, tree_index)
from . import numpy_loader
from .numpy_loader import DeviceNumpyDataLoader, NumpyDataLoader
