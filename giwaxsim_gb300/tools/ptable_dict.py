"""Element tables used by the forward path.

ptable: atomic numbers Z (H..U).  The scattering factor of an atom is
Z + f' + i f'' (tools/comparison.py:735-739 of the reference).

aff_dict: Cromer-Mann coefficients (a1, b1, a2, b2, a3, b3, a4, b4, c) of
International Tables for Crystallography Vol. C, Table 6.1.1.4, for
f0(q) = sum_i a_i exp(-b_i (q/4pi)^2) + c.  The reference's I(q) epilogue
(tools/voxelgrids.py:828-857, called with 'C' at tools/comparison.py:785)
uses carbon; other elements can be added with their published coefficients.
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
}
