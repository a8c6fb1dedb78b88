"""stile_gb300: hybrid sparse-tile SpMM / SDDMM for GB300 (sm_103a).

Planning (tile generation, greedy + withdraw search over a cost model) runs
on the host; packed plans run as fused sm_103a kernels: ELL row-bucket tiles
on CUDA cores, dense 16-row block tiles on the tensor cores (tcgen05, TMEM
accumulators).
"""
from .plan import Plan, Tile, OpSpace  # noqa: F401
from .cost_model import A100_FP16, CostModel, gb300_model  # noqa: F401
from .planner import search_spmm, search_sddmm, estimate_max_bucket_size  # noqa: F401

__all__ = ["Plan", "Tile", "OpSpace", "CostModel", "A100_FP16", "gb300_model", "search_spmm", "search_sddmm",
           "plan_spmm", "plan_sddmm", "spmm", "sddmm", "HybridSpMMFunction", "PlanConfig", "SpmmOperator",
           "SddmmOperator"]


def __getattr__(name):
    # the GPU-facing API imports torch; load it on first use
    if name in ("plan_spmm", "plan_sddmm", "spmm", "sddmm", "HybridSpMMFunction", "PlanConfig",
                "SpmmOperator", "SddmmOperator", "Op", "greedy_search_use_cost_model_lower_bound",
                "post_process_for_withdraw", "measure_seleted_formats", "measure_latency"):
        from . import api
        return getattr(api, name)
    raise AttributeError(name)
