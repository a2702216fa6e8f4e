def print(*a, **k):
    pass
