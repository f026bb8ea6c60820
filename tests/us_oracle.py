"""CPU restatement of the multi-window umbrella-sampling driver, for checking
the engine's US loop.  Test infrastructure only.

Follows MWUSGCMCSimulation / PTMWUSGCMCSimulation (src/us_simulation.cpp:
454-864) with the SimpleUSGCMCSimulation updates (:262-434): per-step visit
counts of the grid order parameter, reweighting by the running biases,
bias = ln p for visited points, -max_D for points seen only before, changes
limited to max_D; neighbouring windows of parity swap_i % 2 exchange when
both points lie in the other window, probability min(1, exp(bias diff)),
drawn from Philox stream 2 keyed (seed, 0).  Window assignments move between
replicas; configurations stay.  The grid order parameter here is the number
of fully bound domains (trace column 3)."""
import math

import numpy as np

from oracle_lib import OracleReplica, set_window, uniform


class USOracle:
    def __init__(self, inp, seed, windows, grid_tag, window_tag, grid_len):
        self.nw = len(windows)
        self.windows = windows
        self.seed = seed
        self.grid_tag = grid_tag
        self.window_tag = window_tag
        self.len = grid_len
        self.reps = [OracleReplica(inp, seed=seed, replica=r) for r in range(self.nw)]
        self.window_of = list(range(self.nw))
        self.replica_of = list(range(self.nw))
        self.E = [np.zeros(grid_len) for _ in range(self.nw)]
        self.inS = [np.zeros(grid_len, bool) for _ in range(self.nw)]
        self.draws = 0
        self.att = [0] * max(self.nw - 1, 1)
        self.acc = [0] * max(self.nw - 1, 1)
        self.apply()

    def apply(self):
        for r, rep in enumerate(self.reps):
            w = self.window_of[r]
            if self.window_tag:
                set_window(rep, self.window_tag, *self.windows[w])
            rep.set_grid(self.grid_tag, self.E[w])

    def run_steps(self, steps, hist):
        for r, rep in enumerate(self.reps):
            tr = rep.run(steps)
            if hist is not None:
                w = self.window_of[r]
                for x in tr[:, 3].astype(int):
                    if 0 <= x < self.len:
                        hist[w][x] += 1

    def exchange(self, swap_i):
        point = [int(self.reps[self.replica_of[w]].observables()["num_fully_bound"]) for w in range(self.nw)]
        self.exchange_points(point, swap_i)
        self.apply()

    def exchange_points(self, point, swap_i):
        """PTMWUSGCMCSimulation::attempt_exchange (:770-864) on the grid
        points of the windows: pairs (i, i+1) from swap_i % 2, both points
        inside the other window, acceptance min(1, exp(bias differences))
        with a draw only when it is not 1 and the points differ."""
        for i in range(swap_i % 2, self.nw - 1, 2):
            self.att[i] += 1
            w1, w2 = i, i + 1
            p1, p2 = point[w1], point[w2]
            lo1, hi1 = self.windows[w1]
            lo2, hi2 = self.windows[w2]
            if p2 < lo1 or p2 > hi1 or p1 < lo2 or p1 > hi2:
                continue
            accepted = True
            if p1 != p2:
                d1 = self.E[w1][p1] - self.E[w2][p1]
                d2 = self.E[w2][p2] - self.E[w1][p2]
                pa = min(1.0, math.exp(d1 + d2))
                if pa != 1:
                    accepted = pa > uniform(self.seed, 0, 2, self.draws)
                    self.draws += 1
            if accepted:
                self.acc[i] += 1
                r1, r2 = self.replica_of[w1], self.replica_of[w2]
                self.replica_of[w1], self.replica_of[w2] = r2, r1
                self.window_of[r1], self.window_of[r2] = w2, w1

    def process(self, hist, max_D):
        for w in range(self.nw):
            self.update_window(w, hist[w], max_D)
        self.apply()

    def update_window(self, w, f, max_D):
        """SimpleUSGCMCSimulation::process_iteration (:160) of window w from
        its visit counts f: estimate_current_weights (:286) reweights the
        visited points by the running biases, update_bias (:385) sets
        ln p for them and -max_D for points seen only before, each change
        limited to max_D."""
        E = self.E[w]
        ave = 0.0
        for x in range(self.len):
            if f[x] > 0:
                ave += f[x] * math.exp(E[x])
        p = [0.0] * self.len
        for x in range(self.len):
            if f[x] > 0:
                p[x] = f[x] * math.exp(E[x]) / ave
                self.inS[w][x] = True
        for x in range(self.len):
            if not self.inS[w][x]:
                continue
            old = E[x]
            if p[x] == 0:
                D = -max_D
                nb = old + D
            else:
                nb = math.log(p[x])
                D = nb - old
            upd = nb
            if abs(D) > max_D:
                upd = old + max_D if D > 0 else old - max_D
            E[x] = upd

    def run(self, n_iters, equil_steps, iter_steps, max_D, exchange_interval=0):
        if equil_steps > 0:
            self.run_steps(equil_steps, None)
        for _ in range(n_iters):
            hist = [[0] * self.len for _ in range(self.nw)]
            if exchange_interval > 0:
                for s in range(1, iter_steps // exchange_interval + 1):
                    self.run_steps(exchange_interval, hist)
                    self.exchange(s)
            else:
                self.run_steps(iter_steps, hist)
            self.process(hist, max_D)
