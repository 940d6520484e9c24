"""Headless monitor with PtyLab's DummyMonitor surface (PtyLab/Monitor/Monitor.py:264-300)."""


class DummyMonitor(object):
    objectZoom = 1
    probeZoom = 1
    figureUpdateFrequency = 1000000
    verboseLevel = "low"

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return lambda *a, **k: None
