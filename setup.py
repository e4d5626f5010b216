"""Packaging of the GB300 library: the counterpart of the reference's
python_package/setup.py.  Building compiles libSharedVDBSCAN.so for sm_103a
with nvcc (variantdbscan_gb300/build.py) and installs it in the package's lib/
directory, beside the Python mirror of the reference wrapper:

    python -m pip install --no-build-isolation .

To serve an installed reference package instead, copy the library into it
with ``python -m variantdbscan_gb300.install <vdbscan package directory>``.
"""
from setuptools import setup
from setuptools.command.build_py import build_py


class BuildWithLibrary(build_py):
    def run(self):
        from variantdbscan_gb300 import build
        build.build()
        super().run()


setup(
    name="variantdbscan-gb300",
    version="0.1",
    description="GB300 (sm_103a) VariantDBSCAN: the libVDBSCAN hot path on the GPU",
    packages=["variantdbscan_gb300"],
    package_data={"variantdbscan_gb300": ["lib/libSharedVDBSCAN.so"]},
    python_requires=">=3.10",
    install_requires=["numpy"],
    cmdclass={"build_py": BuildWithLibrary},
)
