"""Import stub for ``pandas`` -- TEST INFRASTRUCTURE ONLY.

The reference imports pandas at module level (READ_physics.py:1, POST_process.py:2) but uses
it only to read mesh / boundary text files and to write Tecplot ASCII files, none of which
the golden-fixture runs call: meshes are handed to the reference's ``Read.pre_process`` as
arrays.  Any use raises, so a run that would need pandas fails loudly instead of silently.
"""


def _unavailable(*args, **kwargs):
    raise NotImplementedError("pandas is not installed; the reference-execution stand-in does not provide it")


read_csv = _unavailable
DataFrame = _unavailable
