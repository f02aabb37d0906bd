"""placeholder"""
__version__ = "0.12"
