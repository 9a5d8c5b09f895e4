"""`QuantrError` (src/error.rs:17-33): every fallible call raises it with the reference's message."""


class QuantrError(Exception):
    def __init__(self, message: str):
        super().__init__(message)
        self.message = message

    def __str__(self) -> str:  # error.rs:21-25 prints in red with a prefix
        return f"\x1b[91m[Quantr Error] {self.message}\x1b[0m "
