"""Minimal import stub for requests.

ProjectQ's cloud backends import requests at package import time; the
simulator tests never make HTTP calls, and the GPU host has no requests
package.  Only the names those modules import are provided."""

from . import compat, exceptions  # noqa: F401


class Session:
    def __init__(self, *args, **kwargs):
        raise RuntimeError("network access is not available in the test environment")
