"""CUDA-graph replay of resident RK4 steps.

A resident evolution's step is one call into ``libbssn_gb300.so`` that
enqueues a few dozen kernels on the current stream and touches only buffers
the object owns.  ``capture(n)`` records ``n`` such steps as one CUDA graph;
``step(k)`` then replays it whenever ``k`` is a multiple of ``n``, so the host
issues one graph launch instead of one launch per kernel.  Capture records the
kernels without running them, so it does not advance the state; a replay runs
exactly the captured kernels on the same buffers, so replayed steps equal
direct ones bit for bit.
"""

from __future__ import annotations

import torch


class GraphSteps:
    """Mixin for resident evolutions whose ``_advance(steps)`` enqueues the
    steps on the current stream without host synchronisation."""

    _graph = None
    _graph_steps = 0
    graph_launches = 0  # library kernel launches recorded in the captured graph

    def capture(self, steps: int = 1) -> None:
        """Record ``steps`` RK4 steps as a CUDA graph for later ``step`` calls."""
        if steps < 1:
            raise ValueError("steps must be positive")
        torch.cuda.synchronize(self.device)
        graph = torch.cuda.CUDAGraph()
        before = self.lib.bssn_launch_count()
        with torch.cuda.graph(graph):
            self._advance(steps)
        self.graph_launches = self.lib.bssn_launch_count() - before
        self._graph, self._graph_steps = graph, int(steps)

    def release_graph(self) -> None:
        """Drop the captured graph; ``step`` enqueues kernels directly again."""
        self._graph, self._graph_steps, self.graph_launches = None, 0, 0

    @property
    def captured(self) -> bool:
        return self._graph is not None

    def step(self, steps: int = 1) -> None:
        """Advance ``steps`` RK4 steps (graph replays when a capture covers them)."""
        if steps < 0:
            raise ValueError("steps must be non-negative")
        if self._graph is not None and steps % self._graph_steps == 0:
            for _ in range(steps // self._graph_steps):
                self._graph.replay()
        elif steps:
            self._advance(steps)
