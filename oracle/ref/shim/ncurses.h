/* ncurses.h -- terminal-display declarations used by the reference's
 * interactive monitors (not on the path); no-op stubs in shim_stubs.c. */
#ifndef ATMREF_NCURSES_SHIM_H
#define ATMREF_NCURSES_SHIM_H
#include <stdio.h>
typedef struct atmref_screen SCREEN;
typedef struct atmref_window WINDOW;
extern WINDOW* stdscr;
#define A_BOLD 0
#define A_BLINK 0
#define COLOR_BLACK 0
#define COLOR_RED 1
#define COLOR_GREEN 2
#define COLOR_YELLOW 3
#define COLOR_BLUE 4
#define COLOR_MAGENTA 5
#define COLOR_CYAN 6
#define COLOR_WHITE 7
#define COLOR_PAIR(n) (n)
#define getmaxyx(w, y, x) ((y) = 24, (x) = 80)
WINDOW* initscr(void);
int endwin(void);
int printw(const char* fmt, ...);
int mvprintw(int y, int x, const char* fmt, ...);
int attron(int a);
int attroff(int a);
int refresh(void);
int clear(void);
int start_color(void);
int init_pair(short p, short f, short b);
SCREEN* newterm(const char* t, FILE* o, FILE* i);
SCREEN* set_term(SCREEN* s);
#endif
