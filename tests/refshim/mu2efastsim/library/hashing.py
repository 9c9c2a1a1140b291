import hashlib


def content_hash(obj):
    return hashlib.sha256(repr(sorted(obj.items()) if isinstance(obj, dict) else obj).encode()).hexdigest()


def file_sha256(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()
