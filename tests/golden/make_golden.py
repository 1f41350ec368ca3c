"""Generate the committed golden fixtures from the reference's own case files.

Run in a container where the CPanel reference tree is mounted (default path
/root/reference, override with CPANEL_REF).  Writes:

  case4412.npz  -- Connor Cases/4412: the 4412.tri mesh (nodes, 1-based tris, ids),
                   the per-panel fields of V1_Mach0.1_alpha5_beta0/surfaceData-0.vtu
                   (doublet, source, potential, velocity, Cp, centroid; 6 significant
                   digits as printed by the reference) and the .CPout summary numbers.

  case4412_wake.npz -- the same case's V1_Mach0.1_alpha5_beta0/wakeData-0.vtu: wake doublet strength and
                   velocity potential per wake panel (6 significant digits) and the panel centroids from
                   the file's points and connectivity.
  case4412AR6.npz -- Connor Cases/4412AR6 (Stability_Derivatives 1 in its .CPin): the mesh and the
                   .CPout numbers, the ten stability derivatives included (5 decimals).
  case4412_spanwise.npz -- the 4412 case's V1_Mach0.1_alpha5_beta0/spanwiseData_Wake1.csv
                   (cpCase::writeSpanwiseData): its lines as text and the 2y/b, Cl, Cdi columns.

The generated files are small and committed; tests never read the reference tree.
Usage: python make_golden.py [4412 | 4412wake | 4412AR6 | 4412span | steadyTest]  (default: all).
"""
import os
import re
import sys

import numpy as np

REF = os.environ.get("CPANEL_REF", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))


def read_tri(path):
    with open(path) as f:
        tok = f.read().split()
    nn, nt = int(tok[0]), int(tok[1])
    k = 2
    nodes = np.array(tok[k:k + 3 * nn], dtype=np.float64).reshape(nn, 3)
    k += 3 * nn
    tris = np.array(tok[k:k + 3 * nt], dtype=np.int64).reshape(nt, 3)
    k += 3 * nt
    ids = np.array(tok[k:k + nt], dtype=np.int32)
    return nodes, tris, ids


def read_vtu_arrays(path):
    txt = open(path).read()
    out = {}
    for m in re.finditer(r'<DataArray type="(\w+)" Name="([^"]+)"(?: NumberOfComponents="(\d+)")? Format="ascii">(.*?)</DataArray>',
                         txt, re.S):
        typ, name, nc, body = m.group(1), m.group(2), m.group(3), m.group(4)
        vals = np.array(body.split(), dtype=np.float64 if typ.startswith("Float") else np.int64)
        if nc and int(nc) > 1:
            vals = vals.reshape(-1, int(nc))
        out[name] = vals
    return out


def read_cpout(path):
    txt = open(path).read()
    cl, cdi = re.search(r"CL = ([-\d.]+)\s+CDi = ([-\d.]+)", txt).groups()
    nums = re.findall(r"^\s+([-\d.]+)\s+([-\d.]+)\s+([-\d.]+)\s*$", txt, re.M)
    body = [float(v) for v in nums[0]]  # CN CA CY
    wind = [float(v) for v in nums[1]]  # CL CD CY
    mom = [float(v) for v in nums[2]]   # Cm Cl Cn
    return dict(CL=float(cl), CDi=float(cdi), body_CN_CA_CY=body, wind_CL_CD_CY=wind, Cm_Cl_Cn=mom)


def read_stability(path):
    """The two rows under CL_alpha ... and CL_beta ...: (CL, CY, Cm, Cl, Cn) per row."""
    txt = open(path).read()
    rows = []
    for head in ("CL_alpha", "CL_beta"):
        m = re.search(head + r"[^\n]*\n\s*([-\d.]+)\s+([-\d.]+)\s+([-\d.]+)\s+([-\d.]+)\s+([-\d.]+)", txt)
        rows.append([float(v) for v in m.groups()])
    return rows


def main_4412ar6():
    case = os.path.join(REF, "Connor Cases", "4412AR6")
    if not os.path.isdir(case):
        sys.exit("reference case folder not found: %s" % case)
    nodes, tris, ids = read_tri(os.path.join(case, "4412AR6.tri"))
    cp = read_cpout(os.path.join(case, "4412AR6.CPout"))
    da, db = read_stability(os.path.join(case, "4412AR6.CPout"))
    np.savez_compressed(
        os.path.join(HERE, "case4412AR6.npz"),
        nodes=nodes, tris=tris.astype(np.int32), ids=ids,
        CL=cp["CL"], CDi=cp["CDi"], body_CN_CA_CY=np.array(cp["body_CN_CA_CY"]),
        wind_CL_CD_CY=np.array(cp["wind_CL_CD_CY"]), Cm_Cl_Cn=np.array(cp["Cm_Cl_Cn"]),
        d_alpha_CL_CY_Cm_Cl_Cn=np.array(da), d_beta_CL_CY_Cm_Cl_Cn=np.array(db),
        V=1.0, alpha=5.0, beta=0.0, mach=0.1, Sref=6.0, bref=6.0, cref=1.0, cg=np.array([0.25, 0.0, 0.0]))
    print("wrote case4412AR6.npz", nodes.shape, tris.shape, cp, da, db)


def main_4412wake():
    case = os.path.join(REF, "Connor Cases", "4412")
    if not os.path.isdir(case):
        sys.exit("reference case folder not found: %s" % case)
    vtu = read_vtu_arrays(os.path.join(case, "V1_Mach0.1_alpha5_beta0", "wakeData-0.vtu"))
    con = vtu["connectivity"].reshape(-1, 3)
    centroid = vtu["Position"][con].mean(axis=1)
    np.savez_compressed(os.path.join(HERE, "case4412_wake.npz"),
                        mu=vtu["Doublet Strengths"].astype(np.float32),
                        phi=vtu["Velocity Potential"].astype(np.float32), centroid=centroid.astype(np.float32))
    print("wrote case4412_wake.npz", con.shape)


def read_cpin(path):
    """The numeric settings of a .CPin file: single values by key, and the first value of
    the list-valued case blocks (Velocity, Angle_of_Attack, Angle_of_Sideslip, Mach_Number)."""
    lines = [ln.strip() for ln in open(path).read().splitlines()]
    out = {}
    for ln in lines:
        m = re.match(r"(\w+) =\s*(\S+)$", ln)
        if m:
            try:
                out[m.group(1)] = float(m.group(2))
            except ValueError:
                pass
    for i, ln in enumerate(lines):
        key = ln.split(" ")[0]
        if key in ("Velocity", "Angle_of_Attack", "Angle_of_Sideslip", "Mach_Number") and i + 2 < len(lines):
            out[key] = float(lines[i + 2])
        if key in ("Vortex_Particle_Wake", "Accelerate_Code", "Time_Step", "Number_of_Timesteps", "Unsteady_Mode",
                   "Stability_Derivatives") and i + 1 < len(lines):
            out[key] = float(lines[i + 1])
    return out


STEADY_PART_STEPS = (3, 4, 5, 10, 20, 40)  # particle states kept (positions, strengths)
STEADY_BODY_STEPS = (1, 2, 3, 10, 40)      # body doublet and source strengths kept


def main_steadytest():
    case = os.path.join(REF, "Connor Cases", "steadyTest")
    if not os.path.isdir(case):
        sys.exit("reference case folder not found: %s" % case)
    nodes, tris, ids = read_tri(os.path.join(case, "steadyTest.tri"))
    cpin = read_cpin(os.path.join(case, "steadyTest.CPin"))
    cp = read_cpout(os.path.join(case, "steadyTest.CPout"))
    res = os.path.join(case, "V1_Mach0.1_alpha10_beta0")
    nsteps = int(cpin["Number_of_Timesteps"])
    counts, arrays = [], {}
    for s in range(1, nsteps + 1):
        v = read_vtu_arrays(os.path.join(res, "particleData-%d.vtu" % s))
        shed = v.get("Time Step Shed", np.zeros(0))
        counts.append(len(shed))
        if s in STEADY_PART_STEPS:
            arrays["part_pos_%d" % s] = v["Position"].astype(np.float32)
            arrays["part_str_%d" % s] = v["Strength"].astype(np.float32)
        if s == nsteps:
            arrays["shed_step"] = shed.astype(np.int16)
    for s in STEADY_BODY_STEPS:
        v = read_vtu_arrays(os.path.join(res, "surfaceData-%d.vtu" % s))
        arrays["mu_%d" % s] = v["Doublet Strengths"].astype(np.float32)
        arrays["sigma_%d" % s] = v["Source Strengths"].astype(np.float32)
    v = read_vtu_arrays(os.path.join(res, "surfaceData-%d.vtu" % nsteps))
    arrays.update(cp_final=v["Cp"].astype(np.float32), vel_final=v["Velocity"].astype(np.float32),
                  phi_final=v["Velocity Potential"].astype(np.float32))
    np.savez_compressed(
        os.path.join(HERE, "steadyTest.npz"),
        nodes=nodes, tris=tris.astype(np.int32), ids=ids, n_particles=np.array(counts, dtype=np.int32),
        part_steps=np.array(STEADY_PART_STEPS), body_steps=np.array(STEADY_BODY_STEPS),
        CL=cp["CL"], CDi=cp["CDi"], body_CN_CA_CY=np.array(cp["body_CN_CA_CY"]),
        wind_CL_CD_CY=np.array(cp["wind_CL_CD_CY"]), Cm_Cl_Cn=np.array(cp["Cm_Cl_Cn"]),
        V=cpin["Velocity"], alpha=cpin["Angle_of_Attack"], beta=cpin["Angle_of_Sideslip"], mach=cpin["Mach_Number"],
        Sref=cpin["S_ref"], bref=cpin["b_ref"], cref=cpin["c_ref"],
        cg=np.array([cpin["X_cg"], cpin["Y_cg"], cpin["Z_cg"]]), accelerate=int(cpin["Accelerate_Code"]),
        dt=cpin["Time_Step"], steps=nsteps, **arrays)
    print("wrote steadyTest.npz", nodes.shape, tris.shape, cp, cpin, counts[-1])


def main_4412span():
    path = os.path.join(REF, "Connor Cases", "4412", "V1_Mach0.1_alpha5_beta0", "spanwiseData_Wake1.csv")
    with open(path) as f:
        lines = f.read().splitlines()
    vals = np.array([[float(v) for v in ln.split(",")] for ln in lines[1:]])
    np.savez_compressed(os.path.join(HERE, "case4412_spanwise.npz"), lines=np.array(lines),
                        y2b=vals[:, 0], cl=vals[:, 1], cdi=vals[:, 2])
    print("wrote case4412_spanwise.npz", vals.shape)


def main():
    which = sys.argv[1:] or ["4412", "4412wake", "4412AR6", "4412span", "steadyTest"]
    if "4412span" in which:
        main_4412span()
    if "steadyTest" in which:
        main_steadytest()
    if "4412AR6" in which:
        main_4412ar6()
    if "4412wake" in which:
        main_4412wake()
    if "4412" not in which:
        return
    case = os.path.join(REF, "Connor Cases", "4412")
    if not os.path.isdir(case):
        sys.exit("reference case folder not found: %s" % case)
    nodes, tris, ids = read_tri(os.path.join(case, "4412.tri"))
    vtu = read_vtu_arrays(os.path.join(case, "V1_Mach0.1_alpha5_beta0", "surfaceData-0.vtu"))
    cp = read_cpout(os.path.join(case, "4412.CPout"))
    centroid = np.stack([vtu["xPosition"], vtu["yPosition"], vtu["zPostition"]], axis=1)
    np.savez_compressed(
        os.path.join(HERE, "case4412.npz"),
        nodes=nodes, tris=tris.astype(np.int32), ids=ids,
        # printed to 6 significant digits by the reference: float32 keeps them exactly enough
        mu=vtu["Doublet Strengths"].astype(np.float32), sigma=vtu["Source Strengths"].astype(np.float32),
        phi=vtu["Velocity Potential"].astype(np.float32), vel=vtu["Velocity"].astype(np.float32),
        cp=vtu["Cp"].astype(np.float32), centroid=centroid.astype(np.float32),
        CL=cp["CL"], CDi=cp["CDi"], body_CN_CA_CY=np.array(cp["body_CN_CA_CY"]),
        wind_CL_CD_CY=np.array(cp["wind_CL_CD_CY"]), Cm_Cl_Cn=np.array(cp["Cm_Cl_Cn"]),
        V=1.0, alpha=5.0, beta=0.0, mach=0.1, Sref=6.0, bref=6.0, cref=1.0, cg=np.array([0.25, 0.0, 0.0]))
    print("wrote case4412.npz", nodes.shape, tris.shape, cp)


if __name__ == "__main__":
    main()
