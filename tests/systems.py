"""Synthetic origami systems in the reference's file formats.

Every system used by the tests and the benchmark is generated here from a
seed: a scaffold laid out as a serpentine of rows on the z=0 plane, staple
types that pair either two neighbouring domains of one row (helix staples) or
the same column of two neighbouring rows (crossover staples), and sequences
drawn uniformly from ACGT with each staple domain the reverse complement of
its scaffold partner.  Files are written with the reference's JSON layout
(system, movetype, order-parameter and bias files) and its key=value .inp
options."""
import json
import os
import random

COMP = {"A": "T", "T": "A", "G": "C", "C": "G"}


def revcomp(s):
    return "".join(COMP[c] for c in reversed(s))


def serpentine(n, row_len):
    """Positions of n scaffold domains in rows of row_len, alternating x direction."""
    pos = []
    for i in range(n):
        r, c = divmod(i, row_len)
        x = c if r % 2 == 0 else row_len - 1 - c
        pos.append([x, r, 0])
    return pos


def staple_pairs(n, row_len=4):
    """Scaffold index pairs bound by each two-domain staple type (n/2 of them).

    Rows of 4: crossovers join columns 0 and 3 of rows 2k and 2k+1, helix
    staples take the middle pair of each row; an odd last row gets two helix
    staples."""
    assert row_len == 4 and n % 4 == 0
    rows = n // 4
    idx = lambda r, x: 4 * r + (x if r % 2 == 0 else 3 - x)
    pairs = []
    for r in range(0, rows - (rows % 2), 2):
        pairs.append((idx(r, 0), idx(r + 1, 0)))
        pairs.append((idx(r, 3), idx(r + 1, 3)))
        pairs.append((idx(r, 1), idx(r, 2)))
        pairs.append((idx(r + 1, 1), idx(r + 1, 2)))
    if rows % 2:
        r = rows - 1
        pairs.append((idx(r, 0), idx(r, 1)))
        pairs.append((idx(r, 2), idx(r, 3)))
    return pairs


def staple_groups_mixed(n, n_three_pairs):
    """Scaffold index groups of a mixed staple set on rows of 4: the first
    n_three_pairs row pairs each get two three-domain staples (a crossover and
    its neighbour along the row, at both ends) and one helix staple in the
    middle of the first row; the remaining row pairs get the four two-domain
    staples of staple_pairs.  Every group's consecutive scaffold domains are
    lattice neighbours in the serpentine layout."""
    assert n % 8 == 0
    rows = n // 4
    idx = lambda r, x: 4 * r + (x if r % 2 == 0 else 3 - x)
    groups = []
    for k, r in enumerate(range(0, rows, 2)):
        if k < n_three_pairs:
            groups.append((idx(r, 0), idx(r + 1, 0), idx(r + 1, 1)))
            groups.append((idx(r, 3), idx(r + 1, 3), idx(r + 1, 2)))
            groups.append((idx(r, 1), idx(r, 2)))
        else:
            groups.append((idx(r, 0), idx(r + 1, 0)))
            groups.append((idx(r, 3), idx(r + 1, 3)))
            groups.append((idx(r, 1), idx(r, 2)))
            groups.append((idx(r + 1, 1), idx(r + 1, 2)))
    return groups


def linear_pairs(n):
    return [(i, i + 1) for i in range(0, n - 1, 2)]


def ring(n):
    """Positions of n scaffold domains around the edge of a square on the z=0
    plane (n a multiple of 4): a closed loop, for cyclic scaffolds."""
    side = n // 4
    pos = []
    for k in range(side):
        pos.append([k, 0, 0])
    for k in range(side):
        pos.append([side, k, 0])
    for k in range(side):
        pos.append([side - k, side, 0])
    for k in range(side):
        pos.append([0, side - k, 0])
    return pos


def make_system(n, pairs, seed, positions, seq_len=16, cyclic=False, orientations=None):
    rng = random.Random(seed)
    scaf_seq = ["".join(rng.choice("ACGT") for _ in range(seq_len)) for _ in range(n)]
    idents = [[i + 1 for i in range(n)]]
    seqs = [scaf_seq]
    for group in pairs:
        idents.append([-(a + 1) for a in group])
        seqs.append([revcomp(scaf_seq[a]) for a in group])
    return {"origami": {
        "cyclic": cyclic,
        "identities": idents,
        "sequences": seqs,
        "configurations": [{"step": 0, "chains": [{
            "index": 0, "identity": 0,
            "positions": positions,
            "orientations": orientations or [[0, 0, 1]] * n}]}]}}


MOVES = {
    "met3": [("Met staple exchange", "MetStapleExchange", "1/3"),
             ("Met staple regrowth", "MetStapleRegrowth", "1/3"),
             ("CB staple regrowth", "CBStapleRegrowth", "1/3")],
    "all4": [("Orientation rotation", "OrientationRotation", "1/4"),
             ("Met staple exchange", "MetStapleExchange", "1/4"),
             ("Met staple regrowth", "MetStapleRegrowth", "1/4"),
             ("CB staple regrowth", "CBStapleRegrowth", "1/4")],
    # the reference's standard moveset (examples/moveset_standard.json layout):
    # staple moves plus conserved-topology recoil-growth scaffold regrowth
    "ctrg": [("Orientation rotation", "OrientationRotation", "2/6"),
             ("Met staple exchange", "MetStapleExchange", "1/6"),
             ("CB staple regrowth", "CBStapleRegrowth", "1/6"),
             ("Contiguous CTRG scaffold regrowth", "CTRGScaffoldRegrowth", "1/6",
              dict(max_num_recoils=1, max_c_attempts=36, max_regrowth=4)),
             ("Non-contiguous CTRG scaffold regrowth", "CTRGJumpScaffoldRegrowth", "1/6",
              dict(max_num_recoils=1, max_c_attempts=36, max_regrowth=4, max_seg_regrowth=2))],
    # two recoils and fewer trial configurations per domain
    "ctrg2": [("Orientation rotation", "OrientationRotation", "1/4"),
              ("Met staple exchange", "MetStapleExchange", "1/4"),
              ("CB staple regrowth", "CBStapleRegrowth", "1/4"),
              ("Contiguous CTRG scaffold regrowth", "CTRGScaffoldRegrowth", "1/4",
               dict(max_num_recoils=2, max_c_attempts=12, max_regrowth=6))],
    # examples/moveset_standard.json of the reference
    "std": [("Orientation rotation", "OrientationRotation", "2/6"),
            ("Met staple exchange", "MetStapleExchange", "1/6"),
            ("CB staple regrowth", "CBStapleRegrowth", "1/6"),
            ("Contiguous CTRG scaffold regrowth", "CTRGScaffoldRegrowth", "1/6",
             dict(max_num_recoils=1, max_c_attempts=36, max_regrowth=12)),
            ("Non-contiguous CTRG scaffold regrowth", "CTRGJumpScaffoldRegrowth", "1/6",
             dict(max_num_recoils=1, max_c_attempts=36, max_regrowth=12, max_seg_regrowth=2))],
    # every scaffold regrowth movetype together
    "ctall": [("Orientation rotation", "OrientationRotation", "2/8"),
              ("Met staple exchange", "MetStapleExchange", "1/8"),
              ("CB staple regrowth", "CBStapleRegrowth", "1/8"),
              ("Contiguous CTRG scaffold regrowth", "CTRGScaffoldRegrowth", "1/8",
               dict(max_num_recoils=1, max_c_attempts=36, max_regrowth=5)),
              ("Non-contiguous CTRG scaffold regrowth", "CTRGJumpScaffoldRegrowth", "1/8",
               dict(max_num_recoils=1, max_c_attempts=36, max_regrowth=5, max_seg_regrowth=2)),
              ("Contiguous CTCB scaffold regrowth", "CTCBScaffoldRegrowth", "1/8", dict(max_regrowth=5)),
              ("Non-contiguous CTCB scaffold regrowth", "CTCBJumpScaffoldRegrowth", "1/8",
               dict(max_regrowth=5, max_seg_regrowth=2))],
    # scaffold transforms with linker regrowth (src/transform_movetypes.cpp)
    "lkcb": [("Orientation rotation", "OrientationRotation", "2/6"),
             ("Met staple exchange", "MetStapleExchange", "1/6"),
             ("CB staple regrowth", "CBStapleRegrowth", "1/6"),
             ("CTCB linker regrowth", "CTCBLinkerRegrowth", "1/6",
              dict(max_disp=1, max_turns=3, max_regrowth=4, max_linker_length=3, num_transforms=4)),
             ("CTCB clustered linker regrowth", "CTCBClusteredLinkerRegrowth", "1/6",
              dict(max_disp=1, max_turns=3, max_linker_length=3, num_transforms=4))],
    "lkrg": [("Orientation rotation", "OrientationRotation", "2/5"),
             ("Met staple exchange", "MetStapleExchange", "1/5"),
             ("CB staple regrowth", "CBStapleRegrowth", "1/5"),
             ("CTRG linker regrowth", "CTRGLinkerRegrowth", "1/5",
              dict(max_disp=1, max_turns=4, max_regrowth=5, max_linker_length=3, num_transforms=5,
                   max_num_recoils=1, max_c_attempts=36))],
    "lkall": [("Orientation rotation", "OrientationRotation", "2/6"),
              ("Met staple exchange", "MetStapleExchange", "1/6"),
              ("CTCB linker regrowth", "CTCBLinkerRegrowth", "1/6",
               dict(max_disp=2, max_turns=2, max_regrowth=6, max_linker_length=4, num_transforms=6)),
              ("CTCB clustered linker regrowth", "CTCBClusteredLinkerRegrowth", "1/6",
               dict(max_disp=1, max_turns=1, max_linker_length=4, num_transforms=3)),
              ("CTRG linker regrowth", "CTRGLinkerRegrowth", "1/6",
               dict(max_disp=1, max_turns=3, max_regrowth=4, max_linker_length=3, num_transforms=4,
                    max_num_recoils=2, max_c_attempts=12))],
    # conserved-topology configurational-bias scaffold regrowth
    "ctcb": [("Orientation rotation", "OrientationRotation", "2/6"),
             ("Met staple exchange", "MetStapleExchange", "1/6"),
             ("CB staple regrowth", "CBStapleRegrowth", "1/6"),
             ("Contiguous CTCB scaffold regrowth", "CTCBScaffoldRegrowth", "1/6", dict(max_regrowth=4)),
             ("Non-contiguous CTCB scaffold regrowth", "CTCBJumpScaffoldRegrowth", "1/6",
              dict(max_regrowth=4, max_seg_regrowth=2))],
}


def moves_json(kind):
    mts = []
    for entry in MOVES[kind]:
        label, t, f = entry[:3]
        m = {"label": label, "type": t, "freq": f}
        if t == "MetStapleExchange":
            m["adaptive_exchange"] = False
        if len(entry) > 3:
            m.update(entry[3])
        mts.append(m)
    return {"origami": {"movetypes": mts}}


OPS = {"origami": {"order_params": [
    {"label": "Number of bound staples", "tag": "numstaples", "type": "NumStaples", "level": 0},
    {"label": "Number of fully bound domain pairs", "tag": "numfulldomains", "type": "NumBoundDomainPairs", "level": 0},
    {"label": "Number of misbound domain pairs", "tag": "nummisdomains", "type": "NumMisboundDomainPairs", "level": 0},
    {"label": "Number of stacked domain pairs", "tag": "numstackedpairs", "type": "NumStackedPairs", "level": 0},
    {"label": "Number of linear helices", "tag": "numlinearhelices", "type": "NumLinearHelices", "level": 0},
    {"label": "Number of stacked junctions", "tag": "numstackedjuncts", "type": "NumStackedJuncts", "level": 0},
    {"label": "Bound plus stacked", "tag": "boundplusstacked", "type": "Sum", "ops": ["numfulldomains", "numstackedpairs"], "level": 1},
    {"label": "Staple 1 fully bound", "tag": "st1full", "type": "StapleTypeFullyBound", "staple": 1, "level": 1},
]}}

BIASES = {"origami": {"bias_functions": [
    {"label": "lsw", "tag": "lsw", "type": "LinearStepWell", "min_op": 4, "max_op": 10, "well_bias": 0,
     "min_bias": 2, "slope": 1.5, "ops": ["numfulldomains"], "level": 0},
    {"label": "sq", "tag": "sq", "type": "SquareWell", "min_op": 1, "max_op": 6, "well_bias": -0.5,
     "outside_bias": 1.25, "ops": ["numstaples"], "level": 0},
    {"label": "grid", "tag": "grid", "type": "Grid", "ops": ["numfulldomains"], "level": 0}]}}

# Per-domain order parameters between scaffold domains (DistOrderParam,
# AdjacentSiteOrderParam, src/order_params.cpp:25-133), updated per move, with
# bias functions on them.
OPS_DIST = {"origami": {"order_params": OPS["origami"]["order_params"] + [
    {"label": "End-to-end distance", "tag": "dist0_23", "type": "Dist", "chain1": 0, "domain1": 0, "chain2": 0,
     "domain2": 23, "update_per_domain": False, "level": 0},
    {"label": "Domains 4 and 19 adjacent", "tag": "adj4_19", "type": "AdjacentSite", "chain1": 0, "domain1": 4,
     "chain2": 0, "domain2": 19, "update_per_domain": False, "level": 0},
    {"label": "Distance plus bound", "tag": "distplusbound", "type": "Sum", "ops": ["dist0_23", "numfulldomains"],
     "level": 1}]}}

BIASES_DIST = {"origami": {"bias_functions": [
    {"label": "dist well", "tag": "distwell", "type": "LinearStepWell", "min_op": 2, "max_op": 6, "well_bias": 0,
     "min_bias": 0.5, "slope": 0.75, "ops": ["dist0_23"], "level": 0},
    {"label": "adjacent", "tag": "adj", "type": "SquareWell", "min_op": 1, "max_op": 1, "well_bias": -1.5,
     "outside_bias": 0.0, "ops": ["adj4_19"], "level": 0}]}}

BASE = dict(domain_type="HalfTurn", binding_pot="FourBody", misbinding_pot="Opposing", stacking_pot="Constant",
            hybridization_pot="NearestNeighbour", temp=330, staple_M=1e-6, cation_M=0.5, max_staple_size=2,
            order_parameter_file="ops.json")

# name: (system, moveset, overrides)
CASES = {
    "c1": ("four", "met3", dict(stacking_ene=1000, max_total_staples=4, max_type_staples=4)),
    "g24a": ("grid24", "all4", dict(stacking_ene=-1000, staple_M=1e-3, temp=335, max_total_staples=24,
                                    max_type_staples=4)),
    "g24b": ("grid24", "all4", dict(domain_type="ThreeQuarterTurn", stacking_ene=-1500, staple_M=1e-3, temp=325,
                                    max_total_staples=24, max_type_staples=4, centering_freq=97,
                                    constraint_check_freq=101, apply_mean_field_cor="true")),
    "g24c": ("grid24", "all4", dict(hybridization_pot="Uniform", binding_h=-60387.1, binding_s=-166.06,
                                    misbinding_pot="Disallowed", stacking_ene=-1000, temp=340, staple_M=1e-5,
                                    max_total_staples=24, max_type_staples=4, bias_functions_file="biases.json",
                                    bias_functions_mult=0.7)),
    "g24d": ("grid24", "all4", dict(stacking_pot="SequenceSpecific", staple_M=1e-3, max_total_staples=24,
                                    max_type_staples=4)),
    "g24e": ("grid24", "met3", dict(stacking_ene=-2000, staple_M=1e-2, temp=315, max_total_staples=24,
                                    max_type_staples=3)),
    # the 48-domain PTMC system's shape: 24 two-domain staple types, NN on random 16-mers, 1 uM
    "c3": ("grid48", "met3", dict(stacking_ene=1000, staple_M=1e-6, temp=340, max_total_staples=48,
                                  max_type_staples=2)),
    # scaffold regrowth (conserved topology): recoil growth and configurational bias
    "s24a": ("grid24", "ctrg", dict(stacking_ene=-1000, staple_M=1e-3, temp=335, max_total_staples=24,
                                    max_type_staples=4)),
    "s24b": ("grid24", "ctrg2", dict(domain_type="ThreeQuarterTurn", stacking_ene=-1500, staple_M=1e-3,
                                     temp=325, max_total_staples=24, max_type_staples=4, centering_freq=97,
                                     constraint_check_freq=101)),
    "s24c": ("grid24", "ctcb", dict(stacking_ene=-1000, staple_M=1e-3, temp=335, max_total_staples=24,
                                    max_type_staples=4, bias_functions_file="biases.json",
                                    bias_functions_mult=0.7)),
    # scaffold transforms with linker regrowth: CTCB and clustered CTCB,
    # CTRG, every linker movetype on the ThreeQuarterTurn grid with biases,
    # and on the cyclic scaffold
    "l24a": ("grid24", "lkcb", dict(stacking_ene=-1000, staple_M=1e-3, temp=335, max_total_staples=24,
                                    max_type_staples=4)),
    "l24b": ("grid24", "lkrg", dict(stacking_ene=-1000, staple_M=1e-3, temp=335, max_total_staples=24,
                                    max_type_staples=4)),
    "l24c": ("grid24", "lkall", dict(domain_type="ThreeQuarterTurn", stacking_ene=-1500, staple_M=1e-3,
                                     temp=325, max_total_staples=24, max_type_staples=4,
                                     bias_functions_file="biases.json", bias_functions_mult=0.7)),
    "l24r": ("ring24", "lkall", dict(stacking_ene=-1000, staple_M=1e-3, temp=330, max_total_staples=24,
                                     max_type_staples=4)),
    # cyclic scaffold (a closed ring), every scaffold movetype
    # Dist / AdjacentSite order parameters with biases on a scaffold that moves
    "d24": ("grid24", "ctrg", dict(stacking_ene=-1000, staple_M=1e-3, temp=335, max_total_staples=24,
                                   max_type_staples=4, order_parameter_file="ops_dist.json",
                                   bias_functions_file="biases_dist.json")),
    "r24": ("ring24", "ctall", dict(stacking_ene=-1000, staple_M=1e-3, temp=330, max_total_staples=24,
                                    max_type_staples=4)),
    # the 96-domain ThreeQuarterTurn design (40 staple types of 2-3 domains,
    # 8 bp domains) with the reference's standard moveset
    "c4": ("mixed96", "std", dict(domain_type="ThreeQuarterTurn", stacking_ene=-1000, staple_M=1e-6, temp=310,
                                  max_total_staples=40, max_type_staples=1, max_staple_size=3)),
    # an 8-domain scaffold small enough for the reference's exact enumeration,
    # capped at one staple per type and two in all, where most weight sits in
    # states with one fully and one partly bound staple (or one staple)
    "e8": ("grid8", "met3", dict(stacking_ene=-1000, staple_M=1e-4, temp=355, max_total_staples=2,
                                 max_type_staples=1)),
    # three-domain staples with misbinding disallowed: the other growth-point
    # enumerator (no misbinding) and overcount calculator (misbinding only)
    # of the reference's exact enumeration
    "m8": ("mixed8", "met3", dict(misbinding_pot="Disallowed", max_staple_size=3, stacking_ene=-1000,
                                  staple_M=1e-4, temp=345, max_total_staples=3, max_type_staples=1)),
    # the 48-domain system's shape with the reference's standard moveset
    "s48": ("grid48", "ctrg", dict(stacking_ene=-1000, staple_M=1e-4, temp=335, max_total_staples=48,
                                   max_type_staples=2)),
}


def system_for(name):
    if name == "four":
        pairs = [(1, 0), (3, 2)]
        return make_system(4, pairs, seed=4, positions=[[i, 0, 0] for i in range(4)])
    if name.startswith("ring"):
        n = int(name[4:])
        return make_system(n, linear_pairs(n), seed=n + 1, positions=ring(n), cyclic=True)
    if name == "mixed8":
        # two rows of four: two three-domain staple types (a crossover and a
        # helix neighbour each) and a two-domain helix type, 8 bp domains,
        # scaffold orientations turning by a half turn per domain
        return make_system(8, staple_groups_mixed(8, 1), seed=808, positions=serpentine(8, 4), seq_len=8,
                           orientations=[[0, 0, 1 - 2 * (i % 2)] for i in range(8)])
    if name == "mixed96":
        # the 96-domain design: 16 three-domain and 24 two-domain staple types, 8 bp domains
        return make_system(96, staple_groups_mixed(96, 8), seed=96, positions=serpentine(96, 4), seq_len=8)
    if name.startswith("grid"):
        n = int(name[4:])
        return make_system(n, staple_pairs(n), seed=n, positions=serpentine(n, 4))
    raise KeyError(name)


def write_inp(path, opts):
    with open(path, "w") as f:
        for k, v in opts.items():
            f.write("%s=%s\n" % (k, v))


def write_case(dirname, name, extra=None):
    """Writes <name>.inp and its input files into dirname; returns the .inp path."""
    sysname, moves, over = CASES[name]
    os.makedirs(dirname, exist_ok=True)
    with open(os.path.join(dirname, sysname + ".json"), "w") as f:
        json.dump(system_for(sysname), f)
    with open(os.path.join(dirname, "moves_%s.json" % moves), "w") as f:
        json.dump(moves_json(moves), f)
    with open(os.path.join(dirname, "ops.json"), "w") as f:
        json.dump(OPS, f)
    with open(os.path.join(dirname, "biases.json"), "w") as f:
        json.dump(BIASES, f)
    with open(os.path.join(dirname, "ops_dist.json"), "w") as f:
        json.dump(OPS_DIST, f)
    with open(os.path.join(dirname, "biases_dist.json"), "w") as f:
        json.dump(BIASES_DIST, f)
    opts = dict(BASE)
    opts["origami_input_filename"] = sysname + ".json"
    opts["movetype_file"] = "moves_%s.json" % moves
    opts.update(over)
    if extra:
        opts.update(extra)
    path = os.path.join(dirname, name + ".inp")
    write_inp(path, opts)
    return path


US_WINDOWS = [(0, 8), (4, 14), (10, 20), (16, 24)]


def write_us_case(d):
    """The multi-window umbrella case: the 24-domain g24a system with a
    square-well window on the number of fully bound domains (tag "win"), a
    grid bias on it (tag "grid") and the windows file of US_WINDOWS."""
    os.makedirs(d, exist_ok=True)
    biases = {"origami": {"bias_functions": [
        {"label": "window", "tag": "win", "type": "SquareWell", "min_op": 0, "max_op": 24, "well_bias": 0,
         "outside_bias": 6.0, "ops": ["numfulldomains"], "level": 0},
        {"label": "grid", "tag": "grid", "type": "Grid", "ops": ["numfulldomains"], "level": 0}]}}
    with open(os.path.join(d, "us_biases.json"), "w") as f:
        json.dump(biases, f)
    with open(os.path.join(d, "us.windows"), "w") as f:
        f.write("win\n" + "".join("%d, %d\n" % w for w in US_WINDOWS))
    return write_case(d, "g24a", extra=dict(bias_functions_file="us_biases.json", windows_file="us.windows",
                                            us_grid_bias_tag="grid", staple_M=1e-2, temp=330))


def write_all(dirname):
    return {name: write_case(dirname, name) for name in CASES}


if __name__ == "__main__":
    import sys
    d = sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(__file__), "data")
    for n, p in write_all(d).items():
        print(n, p)
