"""Tile cost models used by the format search.

Costs are predicted latencies of one "wave" of thread blocks of a tile kind
(the reference's unit: ms per wave of SM_num concurrent tiles,
my_cost_model.py:1290-1335).  Three kinds:

* tensor-core block tiles: a measured lookup table keyed by (16, 32, K),
  separate atomic / owned entries (get_benchmark_cost_,
  my_cost_model.py:639-769);
* ELL row-bucket tiles: roofline throughput from FLOPs and 32-byte sectors,
  then a linear fit (memory_cost_tb_given_tile_sizes_and_poses :517-582,
  ELL_cost_model :808-815, cost_tb_latency_given_ELL_tiles :1176-1214);
* 1D SDDMM chunks: the same roofline-plus-linear-fit form
  (_cost_tb_latency_1D_tiles_given_features :1219-1248).

``A100_FP16`` holds the reference's own calibration (A100, fp16, SM_num 108)
and is what plan-parity tests use.  ``gb300_model`` returns the model
recalibrated from timings of this package's own kernels on a GB300
(``calibrate.py``), falling back to the A100 tables scaled by the measured
bandwidth ratio when no calibration file is present.
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import dataclass, field

import numpy as np


@dataclass
class CostModel:
    name: str
    dsize: int = 16                 # bits per value (16: fp16/bf16, 32: fp32)
    sm_num: int = 108
    # tensor-core SpMM tiles (16, 32, K): cost per wave
    tc_owned: dict = field(default_factory=dict)
    tc_atomic: dict = field(default_factory=dict)
    # tensor-core SDDMM tiles (16, J, K)
    tc_sddmm: dict = field(default_factory=dict)
    # ELL: cost = a1 * x + b1 (owned); * (a2 * x_atomic / x + b2) (atomic)
    ell_owned: tuple = (8.80425616e-08, 4.17697078e-04)
    ell_atomic: tuple = (8.80688635, -7.9094305)
    # 1D SDDMM: cost = a * x + b
    one_d: tuple = (5.40647867e-08, 2.14658164e-04)
    # roofline compute cap used by the fits (FLOP per byte-equivalent)
    tp_cap: float = 78 / 1.555

    # ------------------------------------------------------------------
    def tc_cost(self, K, atomic, penalty=1):
        table = self.tc_atomic if atomic else self.tc_owned
        return table[int(K)] / penalty

    def tc_sddmm_cost(self, J, K=16):
        return self.tc_sddmm[(int(J), int(K))]

    def ell_model(self, x_owned, x_atomic, atomic):
        a1, b1 = self.ell_owned
        a2, b2 = self.ell_atomic
        if atomic:
            return (a1 * x_owned + b1) * (a2 * x_atomic / x_owned + b2)
        return a1 * x_owned + b1

    def ell_costs(self, I, J, K, k_is, atomic):
        """Costs of ELL tiles (I rows x J features x K slots) whose B-row
        footprints (distinct columns, +1 if padded and column 0 is absent)
        are ``k_is``."""
        cls = 32 * 8 / self.dsize
        compute = I * J * K * 2
        mem_A = math.ceil(I * K / cls)
        mem_B = math.ceil(J / cls) * np.asarray(k_is)
        store = math.ceil(J * self.dsize / 256) * I
        mem_owned = mem_A + store + mem_B
        tp_owned = np.minimum(compute / (mem_owned * 32), self.tp_cap)
        if not atomic:
            return self.ell_model(compute / tp_owned, None, False)
        mem_atomic = mem_A + store * 2 + mem_B
        tp_atomic = np.minimum(compute / (mem_atomic * 32), self.tp_cap)
        return self.ell_model(compute / tp_owned, compute / tp_atomic, True)

    def ell_lower_bound(self, tile_shapes):
        """Smallest possible predicted cost per covered element of an owned
        ELL tile (lower_bound_ELL_cost_BSPMM)."""
        best = []
        for I, J, K in tile_shapes:
            compute = I * J * K * 2
            mem = (math.ceil(I * K * self.dsize / 256) + math.ceil(J * self.dsize / 256) * (K // 2 + 1)
                   + I * math.ceil(J * self.dsize / 256))
            tp = min(compute / (mem * 32), self.tp_cap)
            best.append(self.ell_model(compute / tp, None, False) / (I * K * J))
        return min(best)

    def one_d_costs(self, row_nums, col_nums, F, chunk):
        compute = F * chunk * 2
        mem = ((np.asarray(row_nums) + np.asarray(col_nums)) * F + chunk) * self.dsize / 8
        tp = np.minimum(compute / mem, self.tp_cap)
        a, b = self.one_d
        return a * (compute / tp) + b

    def one_d_lower_bound(self, F, max_bucket_size):
        rows = np.concatenate([np.arange(1, n + 1) for n in range(1, max_bucket_size + 1)])
        nnzs = np.repeat(np.arange(1, max_bucket_size + 1), np.arange(1, max_bucket_size + 1))
        cols = nnzs / rows
        c = self.one_d_costs(rows, cols, F, max_bucket_size) / nnzs / F
        return float(np.min(c))

    def with_mlp(self, mlp):
        """A copy that scores ELL tiles with the learned model `mlp`
        (stile_gb300.mlp_cost.MlpCostModel); TC and 1D tiles keep the tables
        and fits."""
        m = CostModel.from_json(self.to_json())
        m.mlp = mlp
        m.name = f"{self.name}+{mlp.name}"
        return m

    def to_json(self):
        d = dict(self.__dict__)
        d.pop("mlp", None)
        d["tc_owned"] = {str(k): v for k, v in self.tc_owned.items()}
        d["tc_atomic"] = {str(k): v for k, v in self.tc_atomic.items()}
        d["tc_sddmm"] = {f"{k[0]},{k[1]}": v for k, v in self.tc_sddmm.items()}
        return json.dumps(d, indent=1)

    @staticmethod
    def from_json(s):
        d = json.loads(s)
        d["tc_owned"] = {int(k): v for k, v in d["tc_owned"].items()}
        d["tc_atomic"] = {int(k): v for k, v in d["tc_atomic"].items()}
        d["tc_sddmm"] = {tuple(int(x) for x in k.split(",")): v for k, v in d["tc_sddmm"].items()}
        d["ell_owned"] = tuple(d["ell_owned"])
        d["ell_atomic"] = tuple(d["ell_atomic"])
        d["one_d"] = tuple(d["one_d"])
        return CostModel(**d)


# The reference's calibration (A100-SXM4, fp16, SM_num 108):
# tensor-core SpMM table my_cost_model.py:672-695, ELL fit :786-800, 1D fit
# :1238-1244, TC SDDMM table :736-761.  Needed verbatim to reproduce the
# reference's plans.
A100_FP16 = CostModel(
    name="a100_fp16_reference",
    dsize=16,
    sm_num=108,
    tc_owned={16: 0.0002922496385872364, 32: 0.00041533440351486205, 48: 0.0005173248425126075,
              64: 0.0006273023784160614, 80: 0.0007631871849298477, 96: 0.0008801279217004776,
              112: 0.0009804800152778625, 128: 0.001063014417886734, 144: 0.0012102656066417695,
              160: 0.001244262307882309},
    tc_atomic={16: 0.0009056255966424942, 32: 0.0010332158952951432, 48: 0.001133260801434517,
               64: 0.0012712959945201873, 80: 0.0014235648512840272, 96: 0.0015714305639266968,
               112: 0.0017159168422222137, 128: 0.0018328575789928437, 144: 0.0021766144037246703,
               160: 0.0021382145583629607},
    tc_sddmm={(16, 16): 0.019077118486166 / 100, (32, 16): 0.027914240956306458 / 100,
              (64, 16): 0.04804608225822449 / 100, (16, 32): 0.026531841605901718 / 100,
              (32, 32): 0.0391475185751915 / 100, (64, 32): 0.06515711545944214 / 100,
              (16, 48): 0.03529728576540947 / 100, (32, 48): 0.05030912533402443 / 100,
              (64, 48): 0.07875583320856094 / 100, (16, 64): 0.044257279485464096 / 100,
              (32, 64): 0.06239231675863266 / 100, (64, 64): 0.10551295429468155 / 100,
              (16, 80): 0.05752832442522049 / 100, (32, 80): 0.07265280187129974 / 100,
              (64, 80): 0.118947833776474 / 100, (16, 96): 0.06372351944446564 / 100,
              (32, 96): 0.08369152247905731 / 100, (64, 96): 0.1488281637430191 / 100,
              (16, 112): 0.07803903520107269 / 100, (32, 112): 0.09360384196043015 / 100,
              (64, 112): 0.15593470633029938 / 100, (16, 128): 0.07907328009605408 / 100,
              (32, 128): 0.10522624105215073 / 100, (64, 128): 0.18569216132164001 / 100},
    ell_owned=(8.80425616e-08, 4.17697078e-04),
    ell_atomic=(8.80688635, -7.9094305),
    one_d=(5.40647867e-08, 2.14658164e-04),
    tp_cap=78 / 1.555,
)

GB300_CALIBRATION = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gb300_cost_model.json")


def gb300_model():
    """The cost model recalibrated on GB300 (see calibrate.py)."""
    if os.path.exists(GB300_CALIBRATION):
        with open(GB300_CALIBRATION) as f:
            return CostModel.from_json(f.read())
    m = CostModel.from_json(A100_FP16.to_json())
    m.name = "a100_fp16_reference_sm152"
    m.sm_num = 152
    return m


GB300_MLP = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gb300_mlp_cost_model.json")


def gb300_mlp_model():
    """The learned ELL-tile model trained on GB300 timings (calibrate_mlp.py)."""
    from .mlp_cost import MlpCostModel
    if not os.path.exists(GB300_MLP):
        raise FileNotFoundError(f"no trained model at {GB300_MLP}: run python -m stile_gb300.calibrate_mlp")
    with open(GB300_MLP) as f:
        return MlpCostModel.from_json(f.read())
