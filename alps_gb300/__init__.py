"""GB300-native dispersion-tensor library for hot magnetised plasmas (the
disp()/root-search hot path of danielver02/ALPS).  See alps_gb300.api."""
__all__ = ["api", "workloads", "sharding"]
