"""Element tables used by the forward path.

ptable: atomic numbers Z (H..U).  The scattering factor of an atom is
Z + f' + i f'' (tools/comparison.py:735-739 of the reference).

aff_dict: Cromer-Mann coefficients (a1, b1, a2, b2, a3, b3, a4, b4, c) of
International Tables for Crystallography Vol. C, Table 6.1.1.4, for
f0(q) = sum_i a_i exp(-b_i (q/4pi)^2) + c.  The reference's I(q) epilogue
(tools/voxelgrids.py:828-857, called with 'C' at tools/comparison.py:785)
uses carbon; the multi-q form factors (tools/voxelgrids.py:650-707) use
every element of the structure.
"""
_SYMBOLS = (
    "H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co "
    "Ni Cu Zn Ga Ge As Se Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb "
    "Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re Os "
    "Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U").split()

ptable = {s: i + 1 for i, s in enumerate(_SYMBOLS)}
inverse_ptable = {z: s for s, z in ptable.items()}

aff_dict = {
    "C": (2.31, 20.8439, 1.02, 10.2075, 1.5886, 0.5687, 0.865, 51.6512,
          0.2156),
    "H": (0.489918, 20.6593, 0.262003, 7.74039, 0.196767, 49.5519, 0.049879,
          2.20159, 0.001305),
    "N": (12.2126, 0.0057, 3.1322, 9.8933, 2.0125, 28.9975, 1.1663, 0.5826,
          -11.529),
    "O": (3.0485, 13.2771, 2.2868, 5.7011, 1.5463, 0.3239, 0.867, 32.9089,
          0.2508),
    "F": (3.5392, 10.2825, 2.6412, 4.2944, 1.517, 0.2615, 1.0243, 26.1476,
          0.2776),
    "Si": (6.2915, 2.4386, 3.0353, 32.3337, 1.9891, 0.6785, 1.541, 81.6937,
           1.1407),
    "S": (6.9053, 1.4679, 5.2034, 22.2151, 1.4379, 0.2536, 1.5863, 56.172,
          0.8669),
}
