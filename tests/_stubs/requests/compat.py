"""Import stub: requests.compat.urljoin."""

from urllib.parse import urljoin  # noqa: F401
