"""Element symbols and atomic numbers (Z = 1..86)."""

SYMBOLS = (
    "H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co "
    "Ni Cu Zn Ga Ge As Se Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb "
    "Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re "
    "Os Ir Pt Au Hg Tl Pb Bi Po At Rn"
).split()

MAX_ELEMENT = len(SYMBOLS)


def symbol_to_number(sym: str) -> int:
    s = sym.strip().capitalize()
    try:
        return SYMBOLS.index(s) + 1
    except ValueError as e:
        raise ValueError(f"unknown element symbol {sym!r}") from e


def number_to_symbol(z: int) -> str:
    return SYMBOLS[int(z) - 1]
