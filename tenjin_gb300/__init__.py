"""GB300-native per-timestep update of Tenjin's multi-material solver.

Modules:

* ``host``: ``TenjinGPU``, the reference's operators over the C ABI of
  ``libtenjin_gpu.so`` (``_lib`` holds the ctypes signatures of
  ``include/tenjin_gpu.h``);
* ``cases``: the synthetic workloads (shock tube, shock-bubble, copper plate,
  uneven 3-D boxes, solid/fluid mixtures, reactive charge) as ``Case``;
* ``settings``: the reference's libconfig input decks mapped onto a ``Case``;
* ``output``: plotfiles and 1-D dumps in the reference's formats, and its
  plotfile cadence;
* ``adjoint``: the forward/backward pair as a ``torch.autograd.Function``;
* ``run``: command-line timing of any workload;
* ``build``: the in-tree nvcc build for sm_103a.
"""
