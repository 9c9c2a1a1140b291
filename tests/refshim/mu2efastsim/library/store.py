class LibraryError(Exception):
    pass
