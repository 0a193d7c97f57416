"""Reader of the response-bispectrum export files bsa_Run writes in visual mode or base export
mode (bsaexport_cls.brm, bsaexport_msh.brm / .brn; the layout of the reference's
exportBRM_base_internal_, src/bsa/BsaLibImpl.F90:1852-1913, unformatted stream: little-endian
int32 header and zone records, float32 points)."""
from __future__ import annotations

import numpy as np


def read(path):
    """dict(nm, modes, ncomb, ispsym, nzones, npts, zones=[dict(id, nI, nJ, f1, f2, values)])."""
    raw = np.fromfile(path, dtype=np.uint8)
    i32 = lambda off: int(np.frombuffer(raw[off:off + 4].tobytes(), dtype="<i4")[0])
    off = 0
    nm = i32(off); off += 4
    modes = np.frombuffer(raw[off:off + 4 * nm].tobytes(), dtype="<i4").copy(); off += 4 * nm
    ncomb, ispsym, nzones, npts = (i32(off + 4 * k) for k in range(4)); off += 16
    zones = []
    for _ in range(nzones):
        zid, nI, nJ = (i32(off + 4 * k) for k in range(3)); off += 12
        n = nI * nJ
        rec = np.frombuffer(raw[off:off + 4 * n * (ncomb + 2)].tobytes(), dtype="<f4").reshape(n, ncomb + 2)
        off += 4 * n * (ncomb + 2)
        zones.append({"id": zid, "nI": nI, "nJ": nJ, "f1": rec[:, 0].copy(), "f2": rec[:, 1].copy(),
                      "values": rec[:, 2:].copy()})
    if off != raw.size:
        raise ValueError(f"{path}: {raw.size - off} bytes after the last zone")
    return {"nm": nm, "modes": modes, "ncomb": ncomb, "ispsym": ispsym, "nzones": nzones, "npts": npts,
            "zones": zones}
