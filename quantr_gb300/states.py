"""State types of quantr (src/circuit/states/): `Qubit`, `ProductState`, `SuperPosition`.

Host-side containers. Ordering follows the reference exactly: a `ProductState` [q0, q1, ..., qn-1]
is the ket |q0 q1 ... qn-1>, and its index in a `SuperPosition` is sum q_w * 2^(n-1-w)
(`binary_basis` / `comp_basis`, product_states.rs:191-215), wire 0 most significant.
"""
from __future__ import annotations

import enum
from typing import Iterator

import numpy as np

from .errors import QuantrError, rust_display_f64

ZERO_MARGIN = 1e-6  # super_positions.rs:18


class Qubit(enum.IntEnum):
    """|0> or |1> (src/circuit/states/qubit.rs)."""

    Zero = 0
    One = 1

    def kronecker_prod(self, other: "Qubit") -> "ProductState":
        return ProductState._unchecked([self, other])


class ProductState:
    """A computational-basis state |q0 q1 ...> (src/circuit/states/product_states.rs)."""

    __slots__ = ("qubits",)

    def __init__(self, qubits):
        self.qubits = [Qubit(q) for q in qubits]

    @staticmethod
    def new(qubits) -> "ProductState":
        if len(qubits) == 0:  # product_states.rs:37-48
            raise QuantrError("The slice of qubits is empty, it needs to at least have one element.")
        return ProductState(qubits)

    @staticmethod
    def _unchecked(qubits) -> "ProductState":
        return ProductState(qubits)

    def get(self, i: int):
        return self.qubits[i] if 0 <= i < len(self.qubits) else None

    def get_qubits(self) -> list[Qubit]:
        return list(self.qubits)

    def get_mut_qubits(self) -> list[Qubit]:
        return self.qubits

    def num_qubits(self) -> int:
        return len(self.qubits)

    def invert_digit(self, place_num: int) -> "ProductState":
        if not 0 <= place_num < self.num_qubits():  # product_states.rs:154-166 (usize: no negatives)
            raise QuantrError(
                f"The position of the binary digit, {place_num}, is out of bounds. The product "
                f"dimension is {self.num_qubits()}, and so the position must be strictly less.")
        self.qubits[place_num] = Qubit(1 - self.qubits[place_num])
        return self

    def kronecker_prod(self, other: Qubit) -> "ProductState":
        return ProductState(self.qubits + [Qubit(other)])

    def insert_qubits(self, qubits, pos) -> None:  # product_states.rs:112-123
        for q, p in zip(qubits, pos):
            self.qubits[p] = Qubit(q)

    def comp_basis(self) -> int:  # product_states.rs:191-201 (64-bit here, not u32)
        v = 0
        for q in self.qubits:
            v = (v << 1) | int(q)
        return v

    @staticmethod
    def from_(value) -> "ProductState":
        """`From<Qubit>` (product_states.rs:241-257): the one-qubit product state."""
        return ProductState([Qubit(value)])

    @staticmethod
    def binary_basis(index: int, basis_size: int) -> "ProductState":  # product_states.rs:205-215
        return ProductState([(index >> (basis_size - 1 - w)) & 1 for w in range(basis_size)])

    def __iter__(self) -> Iterator[Qubit]:
        return iter(self.qubits)

    def __eq__(self, other) -> bool:
        return isinstance(other, ProductState) and self.qubits == other.qubits

    def __hash__(self) -> int:
        return hash(tuple(int(q) for q in self.qubits))

    def __str__(self) -> str:  # product_states.rs:229-239
        return "".join("1" if q else "0" for q in self.qubits)

    def __repr__(self) -> str:
        return f"ProductState(|{self}>)"


def _equal_within_error(num: float, compare: float) -> bool:
    return compare - ZERO_MARGIN < num < compare + ZERO_MARGIN


class SuperPosition:
    """Dense state vector (src/circuit/states/super_positions.rs). `amplitudes` is complex128."""

    __slots__ = ("amplitudes", "product_dim")

    def __init__(self, amplitudes: np.ndarray, product_dim: int):
        self.amplitudes = np.asarray(amplitudes, dtype=np.complex128)
        self.product_dim = int(product_dim)

    # --- constructors -----------------------------------------------------------------------
    @staticmethod
    def new(prod_dimension: int) -> "SuperPosition":
        if prod_dimension == 0:
            raise QuantrError("The number of qubits must be non-zero.")
        a = np.zeros(1 << prod_dimension, dtype=np.complex128)
        a[0] = 1.0
        return SuperPosition(a, prod_dimension)

    @staticmethod
    def new_unchecked(num_qubits: int) -> "SuperPosition":
        a = np.zeros(1 << num_qubits, dtype=np.complex128)
        a[0] = 1.0
        return SuperPosition(a, num_qubits)

    @staticmethod
    def new_with_amplitudes(amplitudes) -> "SuperPosition":
        a = np.asarray(amplitudes, dtype=np.complex128)
        if not _equal_within_error(float(np.sum(np.abs(a) ** 2)), 1.0):
            raise QuantrError("Slice given to set amplitudes in super position does not conserve "
                              "probability, the absolute square sum of the coefficents must be one.")
        n = a.size
        if n == 0 or (n & (n - 1)) != 0:
            raise QuantrError("The length of the array must be of the form 2**n where n is an integer.")
        return SuperPosition(a.copy(), n.bit_length() - 1)

    @staticmethod
    def new_with_amplitudes_unchecked(amplitudes) -> "SuperPosition":
        a = np.asarray(amplitudes, dtype=np.complex128)
        n = a.size
        return SuperPosition(a.copy(), (n & -n).bit_length() - 1)

    @staticmethod
    def new_with_hash_amplitudes(hash_amplitudes: dict) -> "SuperPosition":
        if not hash_amplitudes:
            raise QuantrError("An empty HashMap was given. A superposition must have at least one "
                              "non-zero state.")
        dim = next(iter(hash_amplitudes)).num_qubits()
        total = 0.0
        for st, amp in hash_amplitudes.items():
            if st.num_qubits() != dim:
                raise QuantrError(f"The first state has product dimension of {dim}, whilst the "
                                  f"state, |{st}>, found as a key in the HashMap has dimension "
                                  f"{st.num_qubits()}.")
            total += abs(amp) ** 2
        if not _equal_within_error(total, 1.0):
            raise QuantrError(f"The total sum of the absolute square of all amplitudes, "
                              f"{rust_display_f64(total)}, "
                              "does not equal 1. That is, the superpositon does not conserve "
                              "probability.")
        a = np.zeros(1 << dim, dtype=np.complex128)
        for st, amp in hash_amplitudes.items():
            a[st.comp_basis()] = amp
        return SuperPosition(a, dim)

    @staticmethod
    def from_(value) -> "SuperPosition":
        """`From<ProductState>` / `From<Qubit>` (super_positions.rs:360-393)."""
        if isinstance(value, (Qubit, int)) and not isinstance(value, ProductState):
            value = ProductState([Qubit(value)])
        a = np.zeros(1 << value.num_qubits(), dtype=np.complex128)
        a[value.comp_basis()] = 1.0
        return SuperPosition(a, value.num_qubits())

    # --- accessors -------------------------------------------------------------------------
    def get_amplitude(self, pos: int):
        return complex(self.amplitudes[pos]) if 0 <= pos < self.amplitudes.size else None

    def get_num_qubits(self) -> int:
        return self.product_dim

    def get_dimension(self) -> int:
        return int(self.amplitudes.size)

    def get_amplitudes(self) -> np.ndarray:
        return self.amplitudes

    def get_amplitude_from_state(self, prod_state: ProductState) -> complex:
        if (1 << prod_state.num_qubits()) != self.amplitudes.size:
            raise QuantrError(f"Unable to retreive product state, |\"{prod_state}\"> with dimension "
                              f"{prod_state.num_qubits()}. The superposition is a linear "
                              "combination of states with different dimension. These dimensions "
                              "should be equal.")
        return complex(self.amplitudes[prod_state.comp_basis()])

    def set_amplitudes(self, amplitudes) -> "SuperPosition":
        a = np.asarray(amplitudes, dtype=np.complex128)
        if a.size != self.amplitudes.size:
            raise QuantrError(f"The slice given to set the amplitudes in the computational basis "
                              f"has length {a.size}, when it should have length "
                              f"{self.amplitudes.size}.")
        if not _equal_within_error(float(np.sum(np.abs(a) ** 2)), 1.0):
            raise QuantrError("Slice given to set amplitudes in super position does not conserve "
                              "probability, the absolute square sum of the coefficents must be one.")
        self.amplitudes = a.copy()
        return self

    def set_amplitudes_unchecked(self, amplitudes) -> "SuperPosition":
        self.amplitudes = np.asarray(amplitudes, dtype=np.complex128).copy()
        return self

    def set_amplitudes_from_states(self, amplitudes: dict) -> "SuperPosition":
        if not amplitudes:
            raise QuantrError("An empty HashMap was given. A superposition must have at least one "
                              "non-zero state.")
        total = 0.0
        for st, amp in amplitudes.items():
            if st.num_qubits() != self.product_dim:
                raise QuantrError(f"The first state has product dimension of {self.product_dim}, "
                                  f"whilst the state, |{st}>, found as a key in the HashMap has "
                                  f"dimension {st.num_qubits()}.")
            total += abs(amp) ** 2
        if not _equal_within_error(total, 1.0):
            raise QuantrError("The total sum of the absolute square of all amplitudes does not "
                              "equal 1. That is, the superpositon does not conserve probability.")
        a = np.zeros_like(self.amplitudes)
        for st, amp in amplitudes.items():
            a[st.comp_basis()] = amp
        self.amplitudes = a
        return self

    def to_hash_map(self) -> dict:
        """States with |a|^2 not within 1e-6 of zero (super_positions.rs:315-323)."""
        p = np.abs(self.amplitudes) ** 2
        keep = np.nonzero(~((p > -ZERO_MARGIN) & (p < ZERO_MARGIN)))[0]
        return {ProductState.binary_basis(int(i), self.product_dim): complex(self.amplitudes[i])
                for i in keep}

    def measure(self, u: float | None = None):
        """One shot (super_positions.rs:332-342): first i with u < cumulative |a_i|^2, else None."""
        from . import rng

        if u is None:
            u = rng.next_f64()
        a = self.amplitudes
        # the running sum in index order, one f64 add per amplitude as quantr's loop does
        # (np.cumsum accumulates sequentially); the first i with u < c[i]
        c = np.cumsum(a.real * a.real + a.imag * a.imag)
        i = int(np.searchsorted(c, u, side="right"))
        if i >= c.size:
            return None
        return ProductState.binary_basis(i, self.product_dim)

    def __iter__(self):  # super_position_iter.rs:56-72
        for i, a in enumerate(self.amplitudes):
            yield ProductState.binary_basis(i, self.product_dim), complex(a)

    def __eq__(self, other) -> bool:
        return (isinstance(other, SuperPosition) and self.product_dim == other.product_dim
                and np.array_equal(self.amplitudes, other.amplitudes))

    def __repr__(self) -> str:
        return f"SuperPosition(product_dim={self.product_dim}, amplitudes={self.amplitudes!r})"
