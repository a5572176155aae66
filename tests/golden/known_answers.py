"""Known-answer vectors for the hot path, transcribed from ReaDDy's own unit tests.

Each case names the reference test (file:line) whose inputs and expected outputs it carries.
The CPU oracle is pinned against these (tests/test_oracle_golden.py) and the CUDA path is checked
against the same cases (tests/test_gpu_golden.py).  Forces the reference computes but does not
enforce (its vec3eq calls without REQUIRE) are enforced here.
"""
import math

PI = math.pi

# ---------------------------------------------------------------------------------------------
# pair potentials
# ---------------------------------------------------------------------------------------------
PAIR_CASES = [
    dict(
        name="harmonic_repulsion_two_particles",
        source="readdy/test/TestStateModel.cpp:57-99",
        box=(4., 4., 4.), periodic=(False, False, False), diffusion=(1.0,),
        potentials=[("harmonic_repulsion", 0, 0, dict(k=1.0, d=2.0))],
        positions=[(0., 0., 0.), (0., 0., 1.8)], types=[0, 0],
        energy=0.02,
        forces=[(0, 0, -0.2), (0, 0, 0.2)],
        force_atol=1e-12,
    ),
    dict(
        name="harmonic_repulsion_six_particles",
        source="readdy/test/TestStateModel.cpp:101-181",
        box=(10., 10., 10.), periodic=(True, True, False), diffusion=(1.0, 1.0),
        potentials=[("harmonic_repulsion", 0, 1, dict(k=1.0, d=3.0))],
        positions=[(0, 0, 0), (0, 0.8, 0), (0.2, 0, -0.2), (0, 0, 0.1), (-1.8, -4.0, 1.8), (0.5, 0, 0)],
        types=[0, 0, 0, 1, 1, 1],
        energy=4.205 + 3.125 + 2.4063226755104354 + 2.1148056603830194 + 3.4833346173608031 * 2,
        # per-pair forces of the reference test, combined per particle below
        pair_forces={
            (0, 3): (0, 0, -2.9), (0, 5): (-2.5, 0, 0),
            (1, 3): (0, 2.1768336301410027, -0.27210420376762534),
            (1, 5): (-1.08999682000954, 1.743994912015264, 0),
            (2, 3): (1.4641005886756873, 0, -2.1961508830135306),
            (2, 5): (-2.1961508830135306, 0, -1.4641005886756873),
        },
        force_atol=1e-12,
    ),
    dict(
        name="lennard_jones_3_2",
        source="readdy/test/TestPotentials.cpp:379-447",
        box=(10., 10., 10.), periodic=(True, True, True), diffusion=(1.0,),
        potentials=[("lennard_jones", 0, 0, dict(m=3, n=2, cutoff=1.0, shift=False, epsilon=1.0, sigma=0.1))],
        positions=[(0, 0, 0), (0, 0, .09), (2, 0, 0), (2, 0, .09)], types=[0, 0, 0, 0],
        energy=2.0 * 0.925925925926, energy_rtol=1e-6,
        forces=[(0, 0, -123.45679012), (0, 0, 123.45679012), (0, 0, -123.45679012), (0, 0, 123.45679012)],
        force_atol=1e-6,
    ),
    dict(
        name="screened_electrostatics",
        source="readdy/test/TestPotentials.cpp:448-505",
        box=(10., 10., 10.), periodic=(False, False, False), diffusion=(1.0,),
        potentials=[("screened_electrostatics", 0, 0,
                     dict(C=-1.0, kappa=1.0, D=1.0, sigma=1.0, exponent=6, cutoff=8.0))],
        positions=[(0, 0, 0), (1.2, 1.5, -1.7)], types=[0, 0],
        energy=-0.0264715664281, energy_rtol=1e-9,
        forces=[(0.01565262, 0.01956577, -0.02217454), (-0.01565262, -0.01956577, 0.02217454)],
        force_atol=1e-8,
    ),
]

# ---------------------------------------------------------------------------------------------
# bonded terms of static topologies
# ---------------------------------------------------------------------------------------------
BONDED_CASES = [
    dict(
        name="harmonic_bond",
        source="readdy/test/TestTopologies.cpp:83-128",
        box=(10., 10., 10.), periodic=(True, True, True),
        positions=[(4, 0, 0), (1, 0, 0)],
        bonds=[((0, 1), 10.0, 5.0)], angles=[], dihedrals=[],
        energy=40.0, energy_rtol=0.0,
        forces=[(40., 0, 0), (-40., 0, 0)], force_atol=0.0,
    ),
    dict(
        name="harmonic_angle",
        source="readdy/test/TestTopologies.cpp:130-178",
        box=(10., 10., 10.), periodic=(True, True, True),
        positions=[(0, 0, 0), (1, 0, 0), (1, 1, 0)],
        bonds=[], angles=[((0, 1, 2), 1.0, PI)], dihedrals=[],
        energy=2.4674011002723395, energy_rtol=1e-5,
        forces=[(0, -3.14159265, 0), (-3.14159265, 3.14159265, 0), (3.14159265, 0., 0.)], force_atol=1e-6,
    ),
    dict(
        name="harmonic_angle_general",
        source="readdy/test/TestTopologies.cpp:180-215",
        box=(10., 10., 10.), periodic=(True, True, True),
        positions=[(0.1, 0.1, 0.1), (1.0, 0.0, 0.0), (1.0, 0.5, -.3)],
        bonds=[], angles=[((0, 1, 2), 1.0, PI)], dihedrals=[],
        energy=2.5871244540347655, energy_rtol=1e-5,
        forces=[(-0.13142034, -3.01536661, 1.83258358), (-5.32252362, 3.44312692, -1.11964973),
                (5.45394396, -0.42776031, -0.71293385)], force_atol=1e-6,
    ),
    dict(
        name="cosine_dihedral",
        source="readdy/test/TestTopologies.cpp:217-273",
        box=(10., 10., 10.), periodic=(True, True, True),
        positions=[(-1, 0, 0), (0, 0, 0), (0, 0, 1), (1, .1, 1)],
        bonds=[], angles=[], dihedrals=[((0, 1, 2, 3), 1.0, 3, PI)],
        energy=0.044370223263673791, energy_rtol=1e-5,
        forces=[(0., -0.88371125, 0.), (0., 0.88371125, 0.), (-0.08749616, 0.87496163, 0.),
                (0.08749616, -0.87496163, 0.)], force_atol=1e-6,
    ),
    dict(
        name="cosine_dihedral_steep",
        source="readdy/test/TestTopologies.cpp:275-311",
        box=(10., 10., 10.), periodic=(True, True, True),
        positions=[(-1, 0, 0), (0, 0, 0), (0, 0, 1), (1, 3, 1)],
        bonds=[], angles=[], dihedrals=[((0, 1, 2, 3), 1.0, 3, PI)],
        energy=1.8221921916437787, energy_rtol=1e-5,
        forces=[(0., 1.70762994, 0.), (0., -1.70762994, 0.), (0.51228898, -0.17076299, 0.),
                (-0.51228898, 0.17076299, 0.)], force_atol=1e-6,
    ),
]

# ---------------------------------------------------------------------------------------------
# reactions with rates so large that every candidate fires (deterministic outcomes)
# ---------------------------------------------------------------------------------------------
REACTION_CASES = [
    dict(
        name="fusion_through_periodic_boundary",
        source="readdy/test/TestReactions.cpp:166-189",
        box=(10., 10., 10.), periodic=(True, True, True), diffusion=(0.,),
        reactions=[("fusion", dict(a=0, b=0, c=0, rate=1e16, educt_distance=2.0))],
        positions=[(4.5, 4.5, 4.5), (-4.7, -4.7, -4.7)], types=[0, 0],
        expect_n=1, expect_positions=[(4.9, 4.9, 4.9)], pos_rtol=1e-6,
    ),
    dict(
        name="parallel_gillespie_eleven_particles",
        source="kernels/cpu/test/TestReactions.cpp:250-355",
        box=(10., 10., 30.), periodic=(True, True, False), diffusion=(.25, .25, .25),
        reactions=[("fusion", dict(a=0, b=0, c=0, rate=1e16, educt_distance=1.0)),
                   ("fusion", dict(a=0, b=2, c=0, rate=2.2250738585072014e-308, educt_distance=1.0)),
                   ("fusion", dict(a=0, b=1, c=0, rate=0.0, educt_distance=1.0))],
        positions=[(0, 0, 0), (0, 0, -.7), (0, 0, .7), (0, 0, -1.6), (0, 0, 1.6), (0, 0, 1.7), (0, 0, -1.7),
                   (0, 0, -5), (0, 0, -5.5), (0, 0, 5), (0, 0, 5.5)],
        types=[0, 0, 2, 2, 0, 0, 1, 0, 0, 0, 0],
        expect_n=7,
        # (type, position) of every particle after one step of the handler
        expect_particles=[(1, (0, 0, -1.7)), (2, (0, 0, .7)), (2, (0, 0, -1.6)), (0, (0, 0, -5.25)),
                          (0, (0, 0, -.35)), (0, (0, 0, 1.65)), (0, (0, 0, 5.25))],
        pos_atol=1e-6,
    ),
]

# Michaelis-Menten integration test, readdy/test/IntegrationTests.cpp:30-106:
# <S> over 37,500 steps must lie within 3 % of 665.2.
# order-1 (external) potentials: (kind, type, args in Context.add_<kind> order after the type)
EXTERNAL_CASES = [
    dict(name="spherical_membrane", source="readdy/test/TestPotentials.cpp:168-214",
         box=(10., 10., 10.), periodic=(True, True, True),
         potentials=[("sphere", 0, (1.0, (1., 0., 0.), 3.0, False)), ("sphere", 0, (1.0, (1., 0., 0.), 3.0, True))],
         positions=[(2., 1., 1.), (4., 3., -3.)], types=[0, 0],
         energy=0.803847577293 + 2.41154273188,
         forces=[(0.73205081, 0.73205081, 0.73205081), (-1.26794919, -1.26794919, 1.26794919)], force_atol=1e-6),
    dict(name="spherical_barrier", source="readdy/test/TestPotentials.cpp:216-259",
         box=(10., 10., 10.), periodic=(True, True, True),
         potentials=[("spherical_barrier", 0, (2.0, 0.3, (1.0, 0.9, 1.0), 1.0))],
         positions=[(2.1, 1., 1.), (1.1, 1., 1.)], types=[0, 0],
         energy=1.51432015278, forces=[(9.2539372, 0.84126702, 0.), (0., 0., 0.)], force_atol=1e-5),
    dict(name="cylinder_inclusion", source="readdy/test/TestPotentials.cpp:261-317",
         box=(20., 20., 20.), periodic=(True, True, True),
         potentials=[("cylinder", 0, (4.0, (1., -2., 3.), (0., 0., 1.), 2.0, True))],
         positions=[(-1., -4., 1.), (0., -3., 3.), (1.5, -1., 5.), (4., -2., 8.)], types=[0, 0, 0, 0],
         energy=3.37258300203048,
         forces=[(2.3431457505076203, 2.3431457505076203, 0.), (0., 0., 0.), (0., 0., 0.), (-4., 0., 0.)],
         force_atol=1e-5),
    dict(name="cylinder_exclusion", source="readdy/test/TestPotentials.cpp:319-375",
         box=(20., 20., 20.), periodic=(True, True, True),
         potentials=[("cylinder", 0, (4.0, (1., -2., 3.), (0., 0., 1.), 2.0, False))],
         positions=[(-1., -4., 1.), (0., -3., 3.), (1.5, -1., 5.), (4., -2., 8.)], types=[0, 0, 0, 0],
         energy=2.2420195910160805,
         forces=[(0., 0., 0.), (-1.6568542494923801, -1.6568542494923801, 0.),
                 (0.5 * 3.155417527999327, 3.155417527999327, 0.), (0., 0., 0.)], force_atol=1e-5),
    # worked by hand from geometry::Box / geometry::Capsule (include/readdy/model/geometry.h:77-162)
    dict(name="box_inclusion_and_exclusion", source="geometry.h:77-116 (hand-worked)",
         box=(10., 10., 10.), periodic=(True, True, True),
         potentials=[("box", 0, (10.0, (-1., -1., -1.), (2., 2., 2.), True)),
                     ("box", 1, (10.0, (-1., -1., -1.), (2., 2., 2.), False))],
         positions=[(1.5, 0., -2.), (0.75, 0.125, 0.)], types=[0, 1],
         energy=6.25 + 0.3125, forces=[(-5., 0., 10.), (2.5, 0., 0.)], force_atol=1e-6),
    dict(name="capsule_inclusion", source="geometry.h:118-162 (hand-worked)",
         box=(10., 10., 10.), periodic=(True, True, True),
         potentials=[("capsule", 0, (2.0, (0., 0., 0.), (0., 0., 2.), 4.0, 1.0, True))],
         positions=[(0., 2., 1.), (0., 0., 3.5), (0., 0.5, -1.5)], types=[0, 0, 0],
         energy=1.0 + 0.25, forces=[(0., -2., 0.), (0., 0., -1.), (0., 0., 0.)], force_atol=1e-6),
]

MICHAELIS_MENTEN = dict(
    source="readdy/test/IntegrationTests.cpp:30-106",
    box=(10., 10., 10.), periodic=(True, True, True),
    diffusion=(0.5, 0.5, 0.5, 0.5),   # E, S, ES, P
    k_fwd=0.0023417691399750494, k_back=1.0, k_prod=1.0, educt_distance=1.0, product_distance=1.0,
    n_e=70, n_s=700, dt=8e-3, n_steps=37500, mean_s=665.2, rel_band=0.03,
)


def per_particle_forces(case):
    """Expected per-particle forces; pair_forces (i,j): f are forces on i, -f on j."""
    if "forces" in case:
        return [tuple(map(float, f)) for f in case["forces"]]
    n = len(case["positions"])
    out = [[0.0, 0.0, 0.0] for _ in range(n)]
    for (i, j), f in case["pair_forces"].items():
        for d in range(3):
            out[i][d] += f[d]
            out[j][d] -= f[d]
    return [tuple(v) for v in out]


# ---------------------------------------------------------------------------------------------
# BreakBonds (readdy/test/TestBreakingBonds.cpp): box 10^3 (periodic), kBT 1, species A, B, C of
# TOPOLOGY flavor with D = 1, one topology type, time step 1, harmonic bonds k = 1, l0 = 1 (energy of a
# bond stretched to 2: 1).  Breakable pairs are (type1, type2, threshold energy, rate); rate 1e10 makes
# the coin certain.  `after` lists the expected sizes of the topologies, sorted; `partners` the type
# multiset of the two-particle piece where the test checks it.
# ---------------------------------------------------------------------------------------------
BREAK_BONDS_CASES = [
    dict(name="dimer_low_threshold", source="readdy/test/TestBreakingBonds.cpp:68-98",
         bonds=[(0, 0)], topologies=[dict(positions=[(0, 0, 0), (0, 0, 2)], types=[0, 0], edges=[(0, 1)])],
         rounds=[[(0, 0, 0.9, 1e10)]], after=[1, 1]),
    dict(name="dimer_high_threshold", source="readdy/test/TestBreakingBonds.cpp:100-112",
         bonds=[(0, 0)], topologies=[dict(positions=[(0, 0, 0), (0, 0, 2)], types=[0, 0], edges=[(0, 1)])],
         rounds=[[(0, 0, 1.1, 1e10)]], after=[2]),
    dict(name="trimer_break_AB", source="readdy/test/TestBreakingBonds.cpp:129-172",
         bonds=[(0, 0), (1, 0)],
         topologies=[dict(positions=[(0, 0, -1), (0, 0, 1), (0, 0, 3)], types=[0, 0, 1], edges=[(0, 1), (1, 2)])],
         rounds=[[(0, 1, 0.9, 1e10)]], after=[1, 2], partners=[0, 0]),
    dict(name="trimer_break_AA", source="readdy/test/TestBreakingBonds.cpp:174-195",
         bonds=[(0, 0), (1, 0)],
         topologies=[dict(positions=[(0, 0, -1), (0, 0, 1), (0, 0, 3)], types=[0, 0, 1], edges=[(0, 1), (1, 2)])],
         rounds=[[(0, 0, 0.9, 1e10)]], after=[1, 2], partners=[0, 1]),
    dict(name="trimer_high_threshold", source="readdy/test/TestBreakingBonds.cpp:197-208",
         bonds=[(0, 0), (1, 0)],
         topologies=[dict(positions=[(0, 0, -1), (0, 0, 1), (0, 0, 3)], types=[0, 0, 1], edges=[(0, 1), (1, 2)])],
         rounds=[[(0, 0, 1.1, 1e10), (0, 1, 1.1, 1e10)]], after=[3]),
    dict(name="three_dimers_one_after_the_other", source="readdy/test/TestBreakingBonds.cpp:263-310",
         bonds=[(0, 0), (1, 1), (2, 2)],
         topologies=[dict(positions=[(0, 0, 0), (0, 0, 2)], types=[t, t], edges=[(0, 1)]) for t in (0, 1, 2)],
         rounds=[[(0, 0, 0.9, 1e10)], [(0, 0, 0.9, 1e10), (1, 1, 0.9, 1e10)],
                 [(0, 0, 0.9, 1e10), (1, 1, 0.9, 1e10), (2, 2, 0.9, 1e10)]],
         after=[1, 1, 1, 1, 1, 1]),
]


# ---------------------------------------------------------------------------------------------
# Spatial topology reactions (readdy/test/TestTopologyReactions.cpp:422-680,
# readdy/test/TestTopologyReactionsExternal.cpp:296-380).  Every species is TOPOLOGY flavored with D = 0;
# bonds are (type1, type2, k, l0); reactions are (mode, (t1, tt1), (t2, tt2), (to1, tto1), (to2, tto2),
# rate, radius, min graph distance) with modes in STRMode order (1 TT_FUSION, 2 TT_FUSION_ALLOW_SELF);
# topologies are (topology type, positions, particle types, edges).  `expect` holds what the reference
# test requires after `steps` steps of length dt.
# ---------------------------------------------------------------------------------------------
_NET_CHAINS = [
    [(-1, 0, 0), (0, 0, 0), (1, 0, 0), (2, 0, 0), (3, 0, 0), (4, 0, 0)],
    [(3, 1, 1), (3, 0, 1), (3, -1, 1), (3, -2, 1), (3, -3, 1), (3, -4, 1)],
    [(4, -3, 0), (3, -3, 0), (2, -3, 0), (1, -3, 0), (0, -3, 0), (-1, -3, 0)],
    [(0, -4, 1), (0, -3, 1), (0, -2, 1), (0, -1, 1), (0, 0, 1), (0, 1, 1)],
]
_NET_BONDS = [(0, 1, 0., .01), (1, 2, 0., .01), (1, 1, 0., .01), (1, 3, 0., .01), (0, 3, 0., .01), (2, 3, 0., .01),
              (3, 3, 0., .01)]  # head 0, core 1, tail 2, link 3
TOPOLOGY_REACTION_CASES = [
    dict(name="tt_fusion", source="readdy/test/TestTopologyReactions.cpp:423-476",
         box=(10., 10., 10.), n_types=4, bonds=[(2, 3, 0., .1)],  # X1 0, X2 1, Y 2, Z 3; T 0, T2 1
         reactions=[(1, (0, 0), (1, 0), (2, 1), (3, 1), 1e10, 1.0, 0)],
         topologies=[(0, [(0, 0, 0)], [0], []), (0, [(0, 0, 0)], [1], [])],
         steps=1, dt=1e-3,
         expect=dict(sizes=[2], types_of_topologies=[1], particle_types=[[2, 3]])),
    dict(name="tt_self_fusion", source="readdy/test/TestTopologyReactions.cpp:478-525",
         box=(10., 10., 10.), n_types=3,  # X 0, Y 1, Z 2; T 0, T2 1
         bonds=[(1, 2, 0., .01), (0, 0, 0., .01), (0, 1, 0., .01), (0, 2, 0., .01)],
         reactions=[(2, (0, 0), (0, 0), (1, 1), (2, 1), 1e10, 1.0, 0)],
         topologies=[(0, [(0, 0, -.01), (0, 0, 0), (0, 0, .01)], [0, 0, 0], [(0, 1), (1, 2)])],
         steps=10, dt=1e-3,
         expect=dict(sizes=[3], types_of_topologies=[1], particle_types=[[0, 1, 2]])),
    dict(name="tt_fusion_network_distance_above_16", source="readdy/test/TestTopologyReactions.cpp:527-618",
         box=(30., 30., 30.), n_types=4, bonds=_NET_BONDS,
         reactions=[(2, (1, 0), (1, 0), (3, 0), (3, 0), 1e10, 1.1, 16)],
         topologies=[(0, c, [0, 1, 1, 1, 1, 2], [(i, i + 1) for i in range(5)]) for c in _NET_CHAINS],
         steps=3, dt=1e-3,
         expect=dict(sizes=[24], links=6)),
    dict(name="tt_fusion_network_distance_above_14", source="readdy/test/TestTopologyReactions.cpp:620-680",
         box=(30., 30., 30.), n_types=4, bonds=_NET_BONDS,
         reactions=[(2, (1, 0), (1, 0), (3, 0), (3, 0), 1e10, 1.01, 14)],
         topologies=[(0, c, [0, 1, 1, 1, 1, 2], [(i, i + 1) for i in range(5)]) for c in _NET_CHAINS],
         steps=10, dt=1e-3,
         expect=dict(sizes=[24], links=8)),
    dict(name="attach_topologies", source="readdy/test/TestTopologyReactionsExternal.cpp:296-380",
         box=(15., 15., 15.), n_types=2, bonds=[(0, 0, 1e-8, 1.), (0, 1, 1e-8, 1.), (1, 1, 1e-8, 1.)],  # middle 0, end 1
         reactions=[(1, (1, 0), (1, 0), (0, 0), (0, 0), 1e3, 1.5, 0)],
         topologies=[(0, [(-4 + 3 * i, 0, 0), (-3 + 3 * i, 0, 0), (-2 + 3 * i, 0, 0)], [1, 0, 1], [(0, 1), (1, 2)])
                     for i in range(3)],
         steps=6, dt=1.0,
         expect=dict(sizes=[9], linear=True, end_x=[-4., 4.])),
]
