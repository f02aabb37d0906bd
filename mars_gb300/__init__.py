"""GB300-native MARS forward pass (candidate projection + hinge-knot sweep).

``mars_gb300.mars`` is the drop-in for the reference ``mars`` module's forward
pass (``fit``, ``expand``, ``pprint``); ``mars_gb300.marslib`` mirrors the
reference's ``marslib`` binding over the C ABI declared in
``include/mars_gpu.h``.
"""
__version__ = "0.12"
