"""python -m cuibm_gb300 -caseFolder <folder> [overrides]: the command-line program
(src/cuIBM.cu main) through the Python binding; the compiled one is
cuibm_gb300/_lib/cuibm (built beside the library)."""
import sys

import cuibm_gb300 as cb


def main(argv):
    folder, rest = ".", []
    k = 0
    while k < len(argv):
        if argv[k] == "-caseFolder" and k + 1 < len(argv):
            folder = argv[k + 1]
            k += 2
            continue
        rest.append(argv[k])
        k += 1
    with cb.NavierStokesSolver(folder, rest) as s:
        s.initialise()
        i = s.info
        print("cuibm: %s, %d x %d cells, solver type %d, %d steps of %g" % (folder, i.nx, i.ny, i.solver_type, i.nt,
                                                                            i.dt))
        while not s.finished():
            s.stepTime(1)
            s.writeData()
        print("cuibm: done; last step's iterations: velocity %d, Poisson %d" % s.iterations())
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
