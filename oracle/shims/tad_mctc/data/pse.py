"""Periodic table symbols (Z <-> symbol) and Pauling electronegativities."""
import torch

_SYMBOLS = (
    "H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co "
    "Ni Cu Zn Ga Ge As Se Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb "
    "Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re "
    "Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U Np Pu Am Cm Bk Cf Es "
    "Fm Md No Lr Rf Db Sg Bh Hs Mt Ds Rg Cn Nh Fl Mc Lv Ts Og"
).split()

Z2S = {i + 1: s for i, s in enumerate(_SYMBOLS)}
S2Z = {s: i + 1 for i, s in enumerate(_SYMBOLS)}
S2Z.update({s.upper(): i + 1 for i, s in enumerate(_SYMBOLS)})
S2Z.update({s.lower(): i + 1 for i, s in enumerate(_SYMBOLS)})


def PAULING(device=None, dtype=torch.double):  # noqa: N802
    raise NotImplementedError("Pauling electronegativities are not needed for GFN1.")
