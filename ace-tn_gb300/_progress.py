"""tqdm when installed (as in the reference), else a silent stand-in."""

try:
    from tqdm import tqdm
except ImportError:  # the GPU image ships without tqdm
    class tqdm:  # noqa: N801 - mirrors the tqdm API used here
        def __init__(self, *args, **kwargs):
            pass

        def update(self, n=1):
            pass

        def close(self):
            pass

        @staticmethod
        def write(msg):
            print(msg)
