"""Serving: continuous batching of LLG runs with block-diagonal CG launches."""
from .blockdiag import BlockDiagPlan, BlockSystem, work_bytes  # noqa: F401
from .engine import Result, ServeStats, ServingEngine, estimate_bytes, run_sequential  # noqa: F401
from .workload import Request, serving_requests  # noqa: F401
