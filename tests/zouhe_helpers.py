"""A channel with Zou-He inlet / outlet (flow-over-sphere benchmark style):
velocity nodes on the x = 0 face, pressure nodes on the x = nx-1 face,
bounce-back walls on the y and z faces, bulk inside."""
import numpy as np

BOUNCE, BULK, PRESSURE, VELOCITY = 0, 2, 5, 6
W19 = np.array([1 / 18] * 3 + [1 / 36] * 6 + [1 / 3] + [1 / 18] * 3 + [1 / 36] * 6)


def channel_classes(nx, ny, nz):
    cls = np.full((nz, ny, nx), BULK, np.uint32)
    cls[:, :, 0] = VELOCITY
    cls[:, :, nx - 1] = PRESSURE
    cls[:, 0, :] = BOUNCE
    cls[:, ny - 1, :] = BOUNCE
    cls[0, :, :] = BOUNCE
    cls[nz - 1, :, :] = BOUNCE
    return cls.ravel()


def channel_flags(nx, ny, nz):
    """Packed flags (class in bits 28..31) before the wall mask is computed."""
    return (channel_classes(nx, ny, nz) << np.uint32(28)).astype(np.uint32)


def channel_init(nx, ny, nz, dtype):
    """f = w at rest on the fluid and Zou-He nodes, 0 on the walls."""
    cls = channel_classes(nx, ny, nz)
    f = np.zeros((19, cls.size), np.float64)
    fluid = cls != BOUNCE
    f[:, fluid] = W19[:, None]
    return f.astype(dtype).ravel()
