"""The seeded multi-scene workloads of the batch and batched-differentiation forms.

Each scene is a triangle soup from the library's soup generator (Q_cuda_make_scene
"soup:n=N,seed=S"); its triangle count (log-uniform), square resolution and samples per pixel
are drawn from numpy's default_rng seeded with the scene seed, so a scene list is the same on
every machine.

  BATCH_64        64 scenes, seeds 1..64, 1e3..5e5 triangles, 64^2..1024^2 pixels, 4/16/64 spp
                  (rendered at depth 6)
  BATCH_64_SMALL  64 scenes, seeds 1..64, 1e3..5e4 triangles, 64^2 or 128^2 pixels, 4 spp
  BATCH_DIFF_32   32 scenes, seeds 101..132, 2e3..1e5 triangles, 128^2..512^2 pixels, 8 spp
                  (depth 4, fitted by Adam)
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class BatchWorkload:
    count: int
    seed0: int
    tris: tuple[float, float]
    sizes: tuple[int, ...]
    spps: tuple[int, ...]
    depth: int

    def draws(self) -> list[tuple[int, int, int, int]]:
        """(scene seed, triangle count, resolution, spp) of every scene."""
        out = []
        for i in range(self.count):
            seed = self.seed0 + i
            rng = np.random.default_rng(seed)
            n = int(round(math.exp(rng.uniform(math.log(self.tris[0]), math.log(self.tris[1])))))
            res = int(rng.choice(self.sizes))
            spp = int(rng.choice(self.spps))
            out.append((seed, n, res, spp))
        return out

    def scenes(self, lib=None) -> list:
        """[(Scene, width, height, spp)] built with the library's generator."""
        from .host import make_scene

        return [(make_scene(f"soup:n={n},seed={seed}", lib), res, res, spp) for seed, n, res, spp in self.draws()]


BATCH_64 = BatchWorkload(64, 1, (1e3, 5e5), (64, 128, 256, 512, 1024), (4, 16, 64), 6)
BATCH_64_SMALL = BatchWorkload(64, 1, (1e3, 5e4), (64, 128), (4,), 6)
BATCH_DIFF_32 = BatchWorkload(32, 101, (2e3, 1e5), (128, 256, 512), (8,), 4)
