"""Recording stand-in for skimage.transform.resize (test infrastructure):
returns its input unchanged and appends (input, output_shape, keyword
arguments) to CALLS, so that the reference's crop window and resize options
can be stored as golden data."""

CALLS = []


def resize(image, output_shape, **kwargs):
    CALLS.append((image.copy(), tuple(int(v) for v in output_shape), dict(kwargs)))
    return image.copy()
