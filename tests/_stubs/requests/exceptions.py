"""Import stub: requests.exceptions."""


class RequestException(IOError):
    pass


class HTTPError(RequestException):
    pass
