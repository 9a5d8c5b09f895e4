"""`QuantrError` (src/error.rs:17-33): every fallible call raises it with the reference's message."""
import decimal
import math


class QuantrError(Exception):
    def __init__(self, message: str):
        super().__init__(message)
        self.message = message

    def __str__(self) -> str:  # error.rs:21-25 prints in red with a prefix
        return f"\x1b[91m[Quantr Error] {self.message}\x1b[0m "


# Values inside messages, printed as quantr's `format!` prints them.

def rust_display_f64(x: float) -> str:
    """`{}` of an f64: the fewest digits that read back to the same value, never an exponent
    (2.0 -> "2", 1e-7 -> "0.0000001", -0.0 -> "-0")."""
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    s = format(decimal.Decimal(repr(x)), "f")
    if "." in s:
        s = s.rstrip("0").rstrip(".")
    return s


def rust_debug_f64(x: float) -> str:
    """`{:?}` of an f64: as `{}` with at least one fractional digit, in exponent form without '+'
    or leading zeros ("1e-5", "1.5e16") below 1e-4 and from 1e16."""
    x = float(x)
    if math.isnan(x) or math.isinf(x):
        return rust_display_f64(x)
    a = abs(x)
    if a == 0.0 or 1e-4 <= a < 1e16:
        s = rust_display_f64(x)
        return s if "." in s else s + ".0"
    mant, exp = repr(x).split("e")
    return f"{mant}e{int(exp)}"


def rust_debug_str(s: str) -> str:
    """`{:?}` of a string: double-quoted, with backslash, quote, \\n, \\r, \\t, \\0 and other
    control characters escaped."""
    out = ['"']
    for ch in s:
        o = ord(ch)
        if ch == "\\":
            out.append("\\\\")
        elif ch == '"':
            out.append('\\"')
        elif ch == "\n":
            out.append("\\n")
        elif ch == "\r":
            out.append("\\r")
        elif ch == "\t":
            out.append("\\t")
        elif ch == "\0":
            out.append("\\0")
        elif o < 0x20 or o == 0x7F:
            out.append(f"\\u{{{o:x}}}")
        else:
            out.append(ch)
    out.append('"')
    return "".join(out)
