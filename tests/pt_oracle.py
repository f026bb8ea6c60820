"""CPU restatement of the 1-D parallel-tempering driver, for checking the
engine's in-kernel exchange.  Test infrastructure only.

Follows PTGCMCSimulation::run (src/ptmc_simulation.cpp:106-150): every round
each replica takes its control quantities (update_control_qs: new energy
tables and a full energy recomputation), runs exchange_interval steps, reports
its dependent quantities (update_dependent_qs, :152), and neighbouring control
slots of parity swap_i % 2 attempt an exchange with calc_acceptance_p
(:275-313) summed over staple types 1..S.  Swap decisions draw from Philox
stream 1 keyed (seed, ladder)."""
import math

import numpy as np

from oracle_lib import OracleReplica, staple_counts, swap_uniform


class PTOracle:
    """dim2 = 0: 1-D ladder over params["temps"] (OneDPTGCMCSimulation);
    dim2 > 0: the temps x stacking_mults grid of TwoDPTGCMCSimulation
    (src/ptmc_simulation.cpp:428-560), exchanging T, staple u and stacking."""

    def __init__(self, inp, params, n_ladders, seed, exchange_q=1, dim2=0, reference_initial_controls=False):
        self.dim2 = dim2
        self.n_ladders = n_ladders
        self.seed = seed
        if dim2:
            temps, stacks = list(params["temps"]), list(params["stacking_mults"])
            d1 = len(temps)
            self.n_rungs = d1 * dim2
            R = self.n_rungs
            self.slot = {"temp": [temps[k // dim2] for k in range(R)],
                         "u": [params.get("staple_u_mult", 1.0)] * R, "bias": [1.0] * R,
                         "stack": [stacks[k % dim2] for k in range(R)]}
            exchange_q = 1 | 2 | 8
            self.sets = []
            i_start, j_start, i_incr, j_incr = [0, 0, 1, 0], [0, 0, 0, 1], [2, 1, 2, 1], [1, 2, 1, 2]
            i_end, j_end, rep_incr = [d1 - 1, d1, d1 - 1, d1], [dim2, dim2 - 1, dim2, dim2 - 1], [dim2, 1, dim2, 1]
            for st in range(4):
                pairs = []
                for i in range(i_start[st], i_end[st], i_incr[st]):
                    for j in range(j_start[st], j_end[st], j_incr[st]):
                        a = i * dim2 + j
                        pairs.append((a, a + rep_incr[st], (st % 2) * d1 * dim2 + i * dim2 + j))
                self.sets.append(pairs)
            n_ctr = 2 * d1 * dim2
        else:
            self.n_rungs = len(params["temps"])
            R = self.n_rungs
            self.slot = {"temp": list(params["temps"]), "u": list(params.get("chem_pot_mults", [1.0] * R)),
                         "bias": list(params.get("bias_mults", [1.0] * R)),
                         "stack": list(params.get("stacking_mults", [1.0] * R))}
            self.sets = [[(i, i + 1, i) for i in range(s0, R - 1, 2)] for s0 in (0, 1)]
            n_ctr = R - 1
        self.q = exchange_q
        self.reps = [OracleReplica(inp, seed=seed, replica=r) for r in range(R * n_ladders)]
        self.ctrl = []
        for l in range(n_ladders):
            for k in range(R):
                self.ctrl.append({n: self.slot[n][k] for n in self.slot})
        if reference_initial_controls:
            # initialize_control_qs (OneD :375-392, TwoD :428-470) stores the
            # bias multiplier of slot k at index m_bias_i = 1 of the control
            # vector, the staple-u slot: until a replica's first exchange its
            # staple u multiplier is that bias multiplier (bias_mults[k]; 1 in
            # 2-D) and its bias multiplier 0.  The engine starts from
            # chem_pot_mults (staple_u_mult in 2-D) and bias_mults instead.
            for l in range(n_ladders):
                for k in range(R):
                    c = self.ctrl[l * R + k]
                    c["u"], c["bias"] = self.slot["bias"][k], 0.0
        self.perm = [[l * R + k for k in range(R)] for l in range(n_ladders)]
        self.draws = [0] * n_ladders
        self.swap_i = 0
        temp0 = params.get("temp", 300.0)
        staple_M = params["staple_M"]
        self.red_u = []
        for n in params["staple_lengths"]:
            extra = (2 * n - 1) * math.log(6)
            u = temp0 * (math.log(staple_M) - extra)
            self.red_u.append(u / temp0)
        self.bias_mult = params.get("bias_functions_mult", 1.0)
        self.att = [0] * n_ctr
        self.acc = [0] * n_ctr

    def round(self, exchange_interval):
        """One PTGCMCSimulation::run round (:106-150): every replica takes its
        controls and runs exchange_interval steps, then every ladder's master
        attempts the exchanges of this round's pair set."""
        self.swap_i += 1
        deps = self.run_interval(exchange_interval)
        for l in range(self.n_ladders):
            self.exchange(l, deps)

    def run_interval(self, exchange_interval):
        """update_control_qs (new energy tables and a full recomputation), the
        steps, then update_dependent_qs (:152): per replica (H, stacking,
        bias, staple counts by type) with counts[0] unused."""
        deps = []
        for r, rep in enumerate(self.reps):
            c = self.ctrl[r]
            rep.update_temp(c["temp"], c["stack"] if self.q & 8 else 1.0)
            rep.run(exchange_interval, trace=False)
            H, S, st, bias = rep.dependent_qs()
            deps.append((H, st, bias, staple_counts(rep)))
        return deps

    def pairs(self):
        """(slot a, slot b, counter) tried this round, in the reference's
        loop order."""
        return self.sets[self.swap_i % len(self.sets)]

    def staple_u(self, r, t):
        """Staple chemical potential of type t (1..S) of replica r:
        update_staple_us, m_reduced_staple_us[t-1] * T * u_mult
        (src/origami_system.cpp:624)."""
        return self.red_u[t - 1] * self.ctrl[r]["temp"] * self.ctrl[r]["u"]

    def acceptance(self, i, i2, r1, r2, deps):
        """calc_acceptance_p (src/ptmc_simulation.cpp:275-313) of exchanging
        the replicas r1 at slot i and r2 at slot i2, summed over staple types
        1..S."""
        t1, t2 = self.slot["temp"][i], self.slot["temp"][i2]
        sm1, sm2 = self.slot["stack"][i], self.slot["stack"][i2]
        H1, st1, b1, n1 = deps[r1]
        H2, st2, b2, n2 = deps[r2]
        dbu = 0.0
        for t in range(1, len(n1)):
            u1 = self.staple_u(r1, t)
            u2 = self.staple_u(r2, t)
            dbu += (u2 / t2 - u1 / t1) * (float(n2[t]) - float(n1[t]))
        DB = 1 / t2 - 1 / t1
        DH = H2 * t2 - H1 * t1
        Dst = st2 * t2 - st1 * t1
        DBM = sm2 / t2 - sm1 / t1
        DBias = b2 * t2 - b1 * t1
        return min(1.0, math.exp(DB * (DH + DBias) + DBM * Dst - dbu))

    def exchange(self, l, deps):
        """attempt_exchange of ladder l (OneD :360-412, TwoD :495-560):
        acceptance draws only when p != 1 (test_acceptance, :262), then
        master_send (:212): each replica takes the controls of its slot."""
        perm = self.perm[l]
        for i, i2, ctr in self.pairs():
            self.att[ctr] += 1
            r1, r2 = perm[i], perm[i2]
            p = self.acceptance(i, i2, r1, r2, deps)
            if p == 1:
                accept = True
            else:
                accept = p > swap_uniform(self.seed, l, self.draws[l])
                self.draws[l] += 1
            if accept:
                self.acc[ctr] += 1
                perm[i], perm[i2] = r2, r1
        self.send_controls(l)

    def send_controls(self, l):
        R = self.n_rungs
        perm = self.perm[l]
        for k in range(R):
            c = self.ctrl[perm[k]]
            if self.q & 1:
                c["temp"] = self.slot["temp"][k]
            if self.q & 2:
                c["u"] = self.slot["u"][k]
            if self.q & 4:
                c["bias"] = self.slot["bias"][k]
            if self.q & 8:
                c["stack"] = self.slot["stack"][k]

    def permutation(self):
        return np.array([x for p in self.perm for x in p], np.int32)
