"""Learned warm start for ROF PDHG solves: a U-Net on the tcgen05 tensor
cores proposes (x0, y0), the fused PDHG finishes to the requested gap."""

from opymize_gb300.warmstart.unet import UNet
from opymize_gb300.warmstart.train import (instance, instances, make_dataset, train, predict,
                                           evaluate, evaluate_restart, solve_batch)

__all__ = ["UNet", "instance", "instances", "make_dataset", "train", "predict", "evaluate",
           "evaluate_restart", "solve_batch"]
