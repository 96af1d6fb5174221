"""tressfx_gb300: TressFX strand simulation and SDF collision on GB300 (sm_103a).

The product is the CUDA library ``libtfxgb300.so`` (C ABI: include/tressfx_gb300.h).  This
package builds it (``tressfx_gb300.build``), binds it (``tressfx_gb300._capi``), and offers
Python handles shaped like the reference's host classes (``tressfx_gb300.api``), seeded
synthetic workloads (``tressfx_gb300.synthetic``) and a headless frame driver
(``tressfx_gb300.headless``).
"""
__version__ = "0.1.0"
