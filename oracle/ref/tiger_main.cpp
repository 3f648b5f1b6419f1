// tiger_main.cpp -- TEST INFRASTRUCTURE ONLY (golden-fixture generation).
// The reference's tiger demo (demos/tiger/tiger.cpp) is compiled against the
// recording canvas with its main() renamed cy_tiger_main; the recorder's
// main() calls cy_test_main, which runs the demo.  The demo draws the tiger
// on 64 canvases and writes the first one's pixels to tiger.tga with its own
// TGA writer (tiger.cpp:4333-4345).
int cy_tiger_main();
int cy_test_main(int, char **) { return cy_tiger_main(); }
