"""Version of this package and of the reference it follows."""
__version__ = '0.1.0'
reference_version = '3.1.7'
