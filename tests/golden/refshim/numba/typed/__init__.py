from .typedlist import List  # noqa: F401
