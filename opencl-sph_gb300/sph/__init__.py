"""Python interface of the GB300 SPH pipeline, mirroring the reference's
``sph`` package (scripts/sph/__init__.py): the same functions with the same
arguments, backed by libsph_gb300.so.  ``init_cuda``/``*_cuda`` names are
provided beside the reference's ``*_opencl`` ones.
"""
from . import bindings as bnd


def init_opencl():
    bnd.init_opencl()


def terminate_opencl():
    bnd.terminate_opencl()


init_cuda = init_opencl
terminate_cuda = terminate_opencl


def init_data(config_file):
    """Builds the host store and its device mirror from a .conf file
    (scripts/sph/__init__.py:11-22)."""
    if bnd.load_config(config_file) > 0:
        print("Initialization failed: could not read config file {}".format(config_file))
        return
    try:
        psdata = init_data_cpu(bnd.get_config_section("psdata_specification"))
        psdata_opencl = init_data_opencl(psdata, bnd.get_config_section("opencl_kernel_files"))
    finally:
        bnd.unload_config()
    return psdata, psdata_opencl


def init_data_from_string(spec, kernel_files):
    """As init_data, from the two section texts instead of a file."""
    psdata = init_data_cpu(spec)
    return psdata, init_data_opencl(psdata, kernel_files)


def init_data_from_dict(config):
    """As init_data, from a dict keyed by the .conf section names
    (``psdata_specification``, ``opencl_kernel_files``); a section may be
    its text or a list of its lines.  The reference declares this function
    with an empty body (scripts/sph/__init__.py:25-26)."""
    def section(name):
        if name not in config:
            raise KeyError("init_data_from_dict: config lacks the [{}] section".format(name))
        text = config[name]
        return text if isinstance(text, str) else "\n".join(text)
    return init_data_from_string(section("psdata_specification"), section("opencl_kernel_files"))


def free_data(psdata, psdata_opencl):
    free_data_cpu(psdata)
    free_data_opencl(psdata_opencl)


def init_data_cpu(config_spec_string):
    import ctypes
    psdata = bnd.psdata()
    bnd.build_psdata_from_string(ctypes.byref(psdata), config_spec_string)
    return psdata


def free_data_cpu(psdata):
    import ctypes
    bnd.free_psdata(ctypes.byref(psdata))


def free_data_opencl(psdata_opencl):
    import ctypes
    bnd.free_psdata_opencl(ctypes.byref(psdata_opencl))


def init_data_opencl(psdata, config_kernels):
    import ctypes
    return bnd.create_psdata_opencl(ctypes.byref(psdata), config_kernels)


init_data_cuda = init_data_opencl
free_data_cuda = free_data_opencl
