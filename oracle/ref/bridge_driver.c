/*
 * bridge_driver.c -- test driver for sdmd_gb300/bridge/sdmd_ref_bridge.c, linked
 * with the UNMODIFIED reference sources into oracle/_ref/libsdmd_ref_bridge.so
 * (oracle/ref/Makefile).  It exposes the reference's own set-up and loop so a
 * test can hand state to the bridge and back:
 *
 *   bd_init(argc, argv)  InputData + Prepare()'s set-up (src/SGThread.c:21-46);
 *                        for a continue run (parameter.txt "continue") InputData
 *                        reads savedData.dat with ReadBreakPoint
 *   bd_save()            the reference's own checkpoint writer (SaveData(savedData))
 *   bd_sweep()           Predict over 1..N and CreateCBT (src/SGThread.c:47-62)
 *   bd_tree()            CreateCBT only (continue mode, src/SGThread.c:54-62)
 *   bd_run(n)            SingleThreadRun's loop (src/SGThread.c:75-151) for n
 *                        more executed events
 *
 * Test infrastructure only.  The reference keeps its state in globals, so each
 * process drives one system.
 */
#include "DMD.h"
#include "sdmd_bridge.h"

int sdmd_ref_rand(void) { return rand(); }

int bd_init(int argc, const char **argv) {
    InputData(argc, argv);
    InitializeFiles(NULL, fileList);
    atomList.ptr = (struct AtomStr **)calloc(atomnum + 1, sizeof(struct AtomStr *));
    for (int i = 1; i <= atomnum; i++) atomList.ptr[i] = &atom[i];
    if (strcmp("new", neworcontinue)) return strcmp("continue", neworcontinue) ? 2 : 0;
    SDEnergyMin(20000, &atomList);
    PBC("full", NULL, &atomList);
    LinkList("full", NULL, NULL, &atomList);
    return 0;
}

void bd_sweep(void) {
    int *renew = calloc(atomnum + 2, sizeof(int));
    for (int i = 1; i <= atomnum; i++) renew[i] = i;
    Predict(renew, &atomList);
    free(renew);
    CreateCBT();
}

void bd_tree(void) { CreateCBT(); }

void bd_save(void) { SaveData(savedData, fileList); }

long bd_run(long n_events) {
    int renewList[256] = {0};
    struct AtomStr *target, *partner;
    const long stop = frame + n_events;
    while (currenttime <= timestep && frame < stop) {
        AssignJob(&target, &partner, renewList, &atomList);
        UpdateData(atomList.timeInr);
        TimeForward(atomList.timeInr);
        currenttime += atomList.timeInr;
        if (!HazardCheck(target, partner, atomList.ptr[target->dynamic->HB.neighbor],
                         partner ? atomList.ptr[partner->dynamic->HB.neighbor] : NULL, &atomList)) {
            frame++;
            DoEvent(&atomList);
            target->dynamic->event.counter++;
            if (renewList[0] == 2 && strcmp(partner->property->extraProperty[1], "_CONS"))
                partner->dynamic->event.counter++;
            Predict(renewList, &atomList);
            UpdateCBT(renewList);
        } else {
            renewList[0] = 1; renewList[2] = 0; renewList[3] = 0;
            Predict(renewList, &atomList);
            UpdateCBT(renewList);
            countReCal++;
        }
    }
    return frame;
}

/* one of the reference's own writers (SaveData, src/DataSave.c:105-160) into its
   output directory, flushed; type is the reference's enum FileType */
void bd_save_type(int type) {
    SaveData((enum FileType)type, fileList);
    if (fileList[type].file) fflush(fileList[type].file);
}
double bd_temperature(void) { return CalSysTem(); }

/* the reference's own energies of its current state (src/ToolFunctions.c:626-752) */
double bd_potential(void) { long w = warningsum; double e = CalPotenE(); warningsum = w; return e; }
double bd_kinetic(void) { return CalKinetE(); }
