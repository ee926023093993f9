"""GB300-native IVF-PQ search engine: a drop-in for the IVF-PQ / PQ search
path of rafaelms101/mestrado (sequential/ivf_pq/ivf_search.cpp,
sequential/pq-utils/pq_search.cpp, parallel2/ivf_pq/mycuda.cu).

The compute runs in hand-written sm_103a CUDA kernels behind the C ABI of
include/gbivf.h; this package holds the build recipe, the ctypes binding,
the host-side index data model, the synthetic input generator and the index
trainer used to make indexes for the benchmark."""
from .ivfdata import IVFPQData  # noqa: F401
from .synth import Mixture  # noqa: F401
